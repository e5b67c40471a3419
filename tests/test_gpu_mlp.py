"""Learned start: features and gradients against the numpy FP64 oracle, and
the effect of a trained network on SCC iterations (the SCC keeps the final
say on the charges)."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu


def test_features_match_oracle(gpu):
    from largetb_gb300 import learned
    m = gpu.model_cristobalite(2, 2, 2, sigma_ang=0.1, seed=9)
    box = learned.cell_box((2, 2, 2))
    f = gpu.mlp_features(m.xyz, m.species, box)
    ref = MO.features(m.xyz, m.species, box)
    np.testing.assert_allclose(f, ref, rtol=1e-5, atol=1e-5)
    assert f.shape == (m.natoms, 32) and f[:, :16].max() > 0.5 and f[:, 16:].max() > 0.5


def test_gradients_match_oracle(gpu):
    from largetb_gb300 import learned
    m = gpu.model_cristobalite(2, 2, 1, sigma_ang=0.1, seed=4)
    X = gpu.mlp_features(m.xyz, m.species, learned.cell_box((2, 2, 1)))
    rng = np.random.default_rng(0)
    Y = rng.normal(0, 0.3, X.shape[0]).astype(np.float32)
    mlp = gpu.MLP(seed=3)
    nrm = np.concatenate([X.mean(0), 1.0 / (X.std(0) + 1e-3)]).astype(np.float32)
    mlp.set(norm=nrm)
    p, _ = mlp.get()
    g, loss = mlp.grad(X, Y)
    gr, lr = MO.grad(p, nrm, X.astype(np.float64), Y.astype(np.float64))
    assert abs(loss - lr) < 1e-5 * max(1.0, lr)
    scale = np.abs(gr).max()
    np.testing.assert_allclose(g, gr, atol=2e-5 * scale, rtol=0)
    y = mlp.predict_fp32(X)  # the training kernels' forward (FP32 layer inputs)
    yr, _ = MO.forward(p, nrm, X.astype(np.float64))
    np.testing.assert_allclose(y, yr, atol=2e-5 * max(1.0, np.abs(yr).max()), rtol=0)


def test_learned_start_cuts_scc_iterations(gpu):
    from largetb_gb300 import learned
    X, Y, _ = learned.dataset(n_cells=32, dims=(2, 2, 2), sigma=(0.02, 0.15), seed=77, M=120, batch=32)
    mlp, loss = learned.train(X, Y, epochs=150, batch=512, lr=3e-3)
    assert loss[-1] < 0.2 * loss[0]
    held = gpu.model_cristobalite(2, 2, 2, sigma_ang=0.09, seed=123456)
    box = learned.cell_box((2, 2, 2))
    q_init = learned.warm_start(mlp, held, box)
    assert abs(q_init.sum() - held.q0.sum()) < 1e-9
    with gpu.Context(M=120, precision=gpu.PREC_FP32) as c:
        c.set_model(held)
        zero = c.scc_solve()
        warm = c.scc_solve(q_init=q_init)
    assert warm["iters"] < zero["iters"]
    assert warm["report"]["dq_max"] < 1e-6
    assert np.abs(warm["q"] - zero["q"]).max() < 3e-6
    err0 = np.abs(held.q0 - zero["q"]).max()
    errw = np.abs(q_init - zero["q"]).max()
    assert errw < 0.5 * err0


def test_tensor_core_forward_matches_oracle(gpu):
    """tb_mlp_predict runs the dense layers on tcgen05 (BF16 layer inputs,
    FP32 accumulation in tensor memory): against the oracle with the same
    BF16 rounding, on a ragged atom count (648 = 5 x 128 + 8); the CUDA-core
    FP32 forward against the FP64 oracle; the shipped weights through both."""
    from largetb_gb300 import learned
    m = gpu.model_cristobalite(3, 3, 3, sigma_ang=0.1, seed=21)
    X = gpu.mlp_features(m.xyz, m.species, learned.cell_box((3, 3, 3)))
    mlp = gpu.MLP(seed=5)
    nrm = np.concatenate([X.mean(0), 1.0 / (X.std(0) + 1e-3)]).astype(np.float32)
    mlp.set(norm=nrm)
    p, _ = mlp.get()
    y_tc, y32 = mlp.predict(X), mlp.predict_fp32(X)
    yb = MO.forward_bf16_inputs(p, nrm, X)
    yr, _ = MO.forward(p, nrm, X.astype(np.float64))
    scale = max(1.0, np.abs(yr).max())
    np.testing.assert_allclose(y_tc, yb, atol=2e-3 * scale, rtol=0)
    np.testing.assert_allclose(y32, yr, atol=2e-5 * scale, rtol=0)
    trained = learned.load()
    a, b = trained.predict(X), trained.predict_fp32(X)
    assert np.abs(a - b).max() < 0.02 and np.abs(a).max() > 0.1
