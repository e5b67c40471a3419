"""SP2 block SpGEMM (tb_sp2) against the FP64 CPU oracle's SP2.

Both run the same recursion: X_0 from Gershgorin, the reference's branch
rule (X^2 if 2 tr X > N_e, else 2X - X^2), 4x4 blocks dropped below the drop
tolerance, the same stopping rule.  FP64 blocks agree with the oracle up to
summation order (charges 1e-8 e without dropping); FP32 blocks stop at their
own idempotency floor, held to charges within 1e-4 e.  At full size both are
also held to the exact projector (dense eigendecomposition).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(nx, ny, nz, sigma=0.08, seed=3003):
    import largetb_gb300 as T
    return (T.model_cristobalite(nx, ny, nz, sigma_ang=sigma, seed=seed),
            O.cristobalite(nx, ny, nz, sigma_ang=sigma, seed=seed))


def _run(T, m, prec, drop=1e-5, max_iter=40):
    with T.Context(precision=prec, sp2_drop_tol=drop, sp2_max_iter=max_iter,
                   sp2_idem_tol=1e-10) as c:
        c.set_model(m)
        return c.sp2()


@pytest.mark.parametrize("drop", [0.0, 1e-5])
def test_sp2_fp64_matches_oracle(gpu, drop):
    m, o = _pair(2, 2, 2)
    ref = O.sp2(o, drop_tol=drop, max_iter=40, idem_tol=1e-10)
    r = _run(gpu, m, gpu.PREC_FP64, drop)
    rep = r["report"]
    assert rep["sp2_iters"] == ref["iters"]
    assert np.abs(r["q"] - ref["q"]).max() < 1e-8
    assert abs(r["e_band"] - ref["e_band"]) < 1e-7
    assert abs(rep["idem_err"] - ref["idem_err"]) < 1e-8
    assert rep["sp2_nnzb"] == ref["nnzb"]


def test_sp2_fp32_matches_oracle(gpu):
    m, o = _pair(2, 2, 2)
    ref = O.sp2(o, drop_tol=1e-5, max_iter=40, idem_tol=1e-10)
    r = _run(gpu, m, gpu.PREC_FP32)
    rep = r["report"]
    assert abs(rep["sp2_iters"] - ref["iters"]) <= 3
    assert rep["idem_err"] < 1e-3
    assert np.abs(r["q"] - ref["q"]).max() < 1e-4
    assert abs(r["q"].sum() - m.n_electrons) < 1e-3
    assert abs(r["e_band"] - ref["e_band"]) / m.natoms < 1e-5


def _exact(cells):
    """The exact zero-temperature density of the SP2 cell (dense FP64
    eigendecomposition, tests/golden/make_sp2_exact.py)."""
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                "sp2_exact_%dx%dx%d.npz" % cells))


def test_sp2_full_size_4x4x4(gpu):
    """1536 atoms, 6144 orbitals, sigma 0.08 A, drop 1e-5, <= 40 steps.

    Against the exact projector (eigendecomposition of H): the 1e-5 drop
    tolerance itself costs 3.7e-5 e in the charges and 3.6e-8 Ha/atom in the
    band energy (the FP64 oracle's own thresholded SP2 lands there), so both
    precisions are held to 1e-4 e and 1e-7 Ha/atom of the exact result, and
    the FP64 blocks to the FP64 oracle's thresholded result within 2e-5 e
    (the drop decisions of blocks near the threshold differ with summation
    order)."""
    m, o = _pair(4, 4, 4)
    ex = _exact((4, 4, 4))
    ref = O.sp2(o, drop_tol=1e-5, max_iter=40, idem_tol=1e-10)
    r64 = _run(gpu, m, gpu.PREC_FP64)
    r32 = _run(gpu, m, gpu.PREC_FP32)
    assert abs(r64["report"]["sp2_iters"] - ref["iters"]) <= 1
    assert np.abs(r64["q"] - ref["q"]).max() < 2e-5
    assert abs(r64["report"]["sp2_nnzb"] - ref["nnzb"]) <= 0.01 * ref["nnzb"]
    assert np.abs(r32["q"] - r64["q"]).max() < 1e-5
    for r in (r64, r32):
        assert abs(r["q"].sum() - m.n_electrons) < 1e-3
        assert r["report"]["idem_err"] < 5e-3
        assert np.abs(r["q"] - ex["q"]).max() < 1e-4
        assert abs(r["e_band"] - float(ex["e_band"])) / m.natoms < 1e-7
        # the symmetric product forms about half of the X^2 block products
        assert 0.4 < r["report"]["sp2_flops_done"] / r["report"]["sp2_flops"] < 0.6


def test_sp2_fp64_tight_drop_reaches_exact(gpu):
    """With the drop tolerance at 1e-7 the FP64 purification reproduces the
    exact projector of the 4x4x4 cell to ~1e-7 e (oracle: 8.4e-8 e): the
    charge error above is the truncation, not the recursion."""
    m, _ = _pair(4, 4, 4)
    ex = _exact((4, 4, 4))
    r = _run(gpu, m, gpu.PREC_FP64, drop=1e-7)
    assert np.abs(r["q"] - ex["q"]).max() < 1e-6
    assert abs(r["e_band"] - float(ex["e_band"])) / m.natoms < 1e-10


def test_density_in_sp2_mode_is_sp2(gpu):
    """tb_params.mode = SP2 routes tb_density to the SP2 solver (same result as
    tb_sp2); the SCC loop stays KPE-only and says so."""
    m = gpu.model_cristobalite(2, 2, 2, sigma_ang=0.08, seed=3003)
    with gpu.Context(precision=gpu.PREC_FP64) as c:
        c.set_model(m)
        ref = c.sp2()
        c.set_params(mode=gpu.MODE_SP2)
        r = c.density()
        # the row accumulator adds with shared-memory atomics: equal to round-off
        np.testing.assert_allclose(r["q"], ref["q"], atol=1e-9, rtol=0)
        assert abs(r["e_band"] - ref["e_band"]) < 1e-9 * m.natoms
        with pytest.raises(gpu.TbError) as e:
            c.scc_solve()
        assert e.value.status == gpu.api.TB_ERR_UNSUPPORTED
