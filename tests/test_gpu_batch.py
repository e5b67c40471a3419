"""Batched SCC (tb_batch_*) against the oracle's SCC of each structure.

Structures of different sizes share every Chebyshev launch but keep their own
scaling, mu, Anderson state and convergence test; each must land where the
oracle's own loop lands (FP32 recurrence: charges within 1e-6 e, iteration
count within 1).  The batch-kernel tests keep every member in the batch
(fp64_small = -1: no FP64 substitution for small members)."""

KEEP = dict(fp64_small=-1)
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [((1, 1, 2), 0.05, 11), ((2, 1, 1), 0.08, 12), ((1, 2, 2), 0.03, 13)]


def test_batch_matches_oracle(gpu):
    models = [gpu.model_cristobalite(*c, sigma_ang=s, seed=sd) for c, s, sd in CASES]
    M = 150
    with gpu.Batch(models, M=M, **KEEP) as b:
        r = b.scc_solve()
    for i, (c, s, sd) in enumerate(CASES):
        o = O.cristobalite(*c, sigma_ang=s, seed=sd)
        ref = O.scc(o, O.kpe_params(M=M, kT=0.01, n_elec=o.n_elec), tol=1e-6, max_iter=100,
                    beta=0.2, history=16)
        assert ref["status"] == 0
        assert abs(int(r["iters"][i]) - ref["iters"]) <= 1, (i, r["iters"][i], ref["iters"])
        assert np.abs(r["q"][i] - ref["q"]).max() < 1e-6
        assert abs(r["e_band"][i] - ref["e_band"]) / o.natoms < 1e-7


def test_batch_agrees_with_single_structure_path(gpu):
    models = [gpu.model_cristobalite(*c, sigma_ang=s, seed=sd) for c, s, sd in CASES]
    with gpu.Batch(models, M=120, **KEEP) as b:
        r = b.scc_solve()
    for i, m in enumerate(models):
        with gpu.Context(M=120, precision=gpu.PREC_FP32, **KEEP) as c:
            c.set_model(m)
            s = c.scc_solve()
        assert abs(int(r["iters"][i]) - s["iters"]) <= 1
        assert np.abs(r["q"][i] - s["q"]).max() < 1e-6


def test_batch_unset_structure_is_reported(gpu):
    m = gpu.model_cristobalite(1, 1, 1, sigma_ang=0.05, seed=1)
    b = gpu.Batch([m], M=50)
    b.close()
    import ctypes as C
    L = gpu.load()
    h = C.c_void_p()
    p = gpu.params(M=50)
    assert L.tb_batch_create(C.byref(p), 2, C.byref(h)) == 0
    rep = gpu.TbReport()
    rc = L.tb_batch_scc_solve(h, None, None, None, None, None, C.byref(rep))
    assert rc == gpu.api.TB_ERR_NOT_READY
    L.tb_batch_destroy(h)


def test_batch_graph_replay_equals_direct_launches(gpu):
    """The batched SCC iteration replayed from graphs captured per active set
    equals launching every kernel directly; a second solve reuses the batch."""
    models = [gpu.model_cristobalite(*c, sigma_ang=s, seed=sd) for c, s, sd in CASES]
    out = {}
    for ng in (0, 1):
        with gpu.Batch(models, M=120, no_graphs=ng, **KEEP) as b:
            r1 = b.scc_solve()
            r2 = b.scc_solve()
        out[ng] = (r1, r2)
    for i in (0, 1):
        a, c = out[0][i], out[1][i]
        np.testing.assert_array_equal(np.asarray(a["iters"]), np.asarray(c["iters"]))
        for qa, qc in zip(a["q"], c["q"]):
            np.testing.assert_array_equal(qa, qc)
        assert a["report"]["kernel_launches"] == c["report"]["kernel_launches"]


def test_batch_pipelined_equals_staged_step(gpu):
    """The batch's pipelined step (persistent CTAs over a tile list of every
    structure's row groups and chunks, bulk copies into a shared-memory ring)
    and its staged step (one CTA per unit) run the same FP32 multiply-add
    chain per block row; only the order in which warps' column sums are added
    differs, so the charges agree far below the FP32 tolerance."""
    models = [gpu.model_cristobalite(*c, sigma_ang=s, seed=sd) for c, s, sd in CASES]
    out = {}
    for kern in (gpu.FP32_STAGED, gpu.FP32_AUTO):
        with gpu.Batch(models, M=120, fp32_kernel=kern, **KEEP) as b:
            out[kern] = b.scc_solve()
    a, c = out[gpu.FP32_STAGED], out[gpu.FP32_AUTO]
    np.testing.assert_array_equal(np.asarray(a["iters"]), np.asarray(c["iters"]))
    for qa, qc in zip(a["q"], c["q"]):
        assert np.abs(qa - qc).max() < 1e-10


def _plus_u(m):
    """The reference's quartz Gamma has -U on the diagonal, under which the
    SCC runs away; the batch tests use +U."""
    g = m.g_vals.copy()
    for a in range(m.natoms):
        for k in range(m.g_rowptr[a], m.g_rowptr[a + 1]):
            if m.g_colidx[k] == a:
                g[k] = -g[k]
    m.g_vals = g
    return m


def _ragged():
    dims = [(1, 1, 1), (2, 1, 1), (3, 3, 1)]
    models = [_plus_u(gpu_mod().model_quartz(*d)) for d in dims]
    models.append(gpu_mod().model_cristobalite(1, 1, 1, sigma_ang=0.05, seed=3))
    oracles = [O.quartz(*d, gamma_diag=1.0) for d in dims] + [O.cristobalite(1, 1, 1, sigma_ang=0.05, seed=3)]
    return models, oracles


def gpu_mod():
    import largetb_gb300 as T
    return T


def test_batch_ragged_tile_lists(gpu):
    """Structures whose atom counts are not multiples of the 24-row groups
    (9, 18 and 81-atom alpha-quartz slabs beside a 24-atom cristobalite
    cell), all kept in the batch's FP32 step: partial last groups and partial
    last chunks in one tile list.  The batch must land where the
    single-structure FP32 path lands.  Both stop at |dq| < 1e-6 e, their
    column sums are added in different orders, and the slabs' SCC response
    amplifies that FP32 rounding noise (~2e-7 e per evaluation) at the fixed
    point, so this FP32-against-FP32 check allows 2e-6 e and 2 iterations.
    Anderson history 4 (16 stored residuals in 9 or 18 dimensions make the
    least-squares step ill-conditioned)."""
    models, _ = _ragged()
    M = 120
    with gpu.Batch(models, M=M, mix_history=4, **KEEP) as b:
        r = b.scc_solve()
    assert r["report"]["fp64_evals"] == 0
    for i, m in enumerate(models):
        with gpu.Context(M=M, precision=gpu.PREC_FP32, mix_history=4, **KEEP) as c:
            c.set_model(m)
            s = c.scc_solve()
        assert abs(int(r["iters"][i]) - s["iters"]) <= 2, (i, r["iters"][i], s["iters"])
        assert np.abs(r["q"][i] - s["q"]).max() < 2e-6, i


def test_batch_small_members_match_oracle(gpu):
    """The same structures with the default settings: members of at most 512
    orbitals (all four here) run the plain FP64 recurrence on their own
    (tb_params.fp64_small), in the batch and in a single FP32 context alike,
    and land where the FP64 oracle's SCC lands -- the reference's own quartz
    geometry to 1e-6 e and 1e-7 Ha/atom, iteration counts within 1."""
    models, oracles = _ragged()
    M = 120
    with gpu.Batch(models, M=M, mix_history=4) as b:
        r = b.scc_solve()
    assert r["report"]["fp64_evals"] > 0
    for i, (m, o) in enumerate(zip(models, oracles)):
        with gpu.Context(M=M, precision=gpu.PREC_FP32, mix_history=4) as c:
            c.set_model(m)
            s = c.scc_solve()
        assert s["report"]["fp64_evals"] == s["iters"]
        ref = O.scc(o, O.kpe_params(M=M, kT=0.01, n_elec=o.n_elec), tol=1e-6, max_iter=100, beta=0.2, history=4)
        assert ref["status"] == 0
        for got in (r["q"][i], s["q"]):
            assert np.abs(got - ref["q"]).max() < 1e-6, i
        for it in (int(r["iters"][i]), s["iters"]):
            assert abs(it - ref["iters"]) <= 1, (i, it, ref["iters"])
        assert abs(r["e_band"][i] - ref["e_band"]) / m.natoms < 1e-7, i
        assert abs(s["e_band"] - ref["e_band"]) / m.natoms < 1e-7, i
