"""CUDA KPE path (through the C-ABI) against the FP64 CPU oracle.

Tolerances: the plain FP64 form must agree with the oracle to round-off
(charges 1e-9 e, band energy 1e-9 Ha); the FP32 form carries the bar of the
task -- charges within 1e-6 e and band energy within 1e-7 Ha/atom.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(nx, ny, nz, sigma=0.05, seed=1001, gamma_diag=1.0):
    import largetb_gb300 as T
    return (T.model_cristobalite(nx, ny, nz, sigma_ang=sigma, seed=seed, gamma_diag=gamma_diag),
            O.cristobalite(nx, ny, nz, sigma_ang=sigma, seed=seed, gamma_diag=gamma_diag))


def _ctx(T, m, **kw):
    # these tests exercise the FP32 kernels on small matrices too: no FP64
    # substitution for small structures (tb_params.fp64_small) unless asked
    kw.setdefault("fp64_small", -1)
    c = T.Context(**kw)
    c.set_model(m)
    return c


@pytest.fixture(scope="module")
def cfg1(gpu):
    """2x2x2 cristobalite, 192 atoms, 768 orbitals, sigma 0.05 A."""
    m, o = _pair(2, 2, 2)
    ref = O.density(o, O.kpe_params(M=200, kT=0.01, n_elec=o.n_elec))
    return m, o, ref


def test_gershgorin_matches_oracle(gpu, cfg1):
    m, o, _ = cfg1
    with _ctx(gpu, m) as c:
        assert np.allclose(c.gershgorin(), O.gershgorin(o), atol=1e-13, rtol=0)
        sh = np.repeat(np.linspace(-0.2, 0.3, m.natoms), 4)
        assert np.allclose(c.gershgorin(sh), O.gershgorin(o, sh), atol=1e-13, rtol=0)


def test_density_fp64_matches_oracle(gpu, cfg1):
    m, o, ref = cfg1
    with _ctx(gpu, m, M=200, precision=gpu.PREC_FP64) as c:
        r = c.density()
    np.testing.assert_allclose(r["moments"], ref["moments"], atol=1e-9 * m.n, rtol=0)
    np.testing.assert_allclose(r["q"], ref["q"], atol=1e-9, rtol=0)
    np.testing.assert_allclose(r["diagP"], ref["diagP"], atol=1e-10, rtol=0)
    assert abs(r["e_band"] - ref["e_band"]) < 1e-9 * m.natoms
    assert abs(r["report"]["n_electrons_found"] - m.n_electrons) < 1e-6
    B = r["report"]["column_block"]
    assert r["report"]["spmm_launches"] == -(-m.n // B) * 200  # M steps per identity slab


def test_density_fp32_matches_oracle(gpu, cfg1):
    m, o, ref = cfg1
    with _ctx(gpu, m, M=200, precision=gpu.PREC_FP32) as c:
        r = c.density()
    assert np.abs(r["q"] - ref["q"]).max() < 1e-6
    assert abs(r["e_band"] - ref["e_band"]) / m.natoms < 1e-7
    np.testing.assert_allclose(r["moments"], ref["moments"], atol=2e-5 * m.n, rtol=0)
    assert abs(r["q"].sum() - m.n_electrons) < 1e-6


@pytest.mark.parametrize("prec", [0, 1])
def test_step_function_and_autocorr_kernel(gpu, prec):
    m, o = _pair(1, 1, 2, seed=7)
    # kT = 0.002: 16384 quadrature nodes read from a cosine table built for 65536
    for kT, kernel in [(0.0, 0), (0.01, 1), (0.02, 2), (0.002, 0)]:
        ref = O.density(o, O.kpe_params(M=120, kT=kT, n_elec=o.n_elec, kernel=kernel))
        with _ctx(gpu, m, M=120, kT=kT, kernel=kernel, precision=prec) as c:
            r = c.density()
        tol = 1e-9 if prec == 0 else 1e-6
        assert np.abs(r["q"] - ref["q"]).max() < tol, (kT, kernel)


@pytest.mark.parametrize("dims", [(1, 1, 1), (1, 1, 3), (1, 2, 3)])
@pytest.mark.parametrize("prec", [0, 1])
def test_ragged_sizes(gpu, dims, prec):
    """n not a multiple of the slab width: padded identity columns."""
    m, o = _pair(*dims, seed=11)
    ref = O.density(o, O.kpe_params(M=80, kT=0.01, n_elec=o.n_elec))
    with _ctx(gpu, m, M=80, precision=prec) as c:
        r = c.density()
    tol = 1e-9 if prec == 0 else 1e-6
    assert np.abs(r["q"] - ref["q"]).max() < tol
    assert np.abs(r["diagP"] - ref["diagP"]).max() < tol


def test_shifted_density_matches_oracle(gpu):
    m, o = _pair(1, 1, 2, seed=3)
    rng = np.random.default_rng(0)
    sh = np.repeat(rng.normal(0, 0.05, m.natoms), 4)
    ref = O.density(o, O.kpe_params(M=100, kT=0.01, n_elec=o.n_elec), shift=sh)
    with _ctx(gpu, m, M=100) as c:
        r = c.density(shift=sh)
    assert np.abs(r["q"] - ref["q"]).max() < 1e-9


def test_coulomb_shift_reference_triple(gpu, golden):
    """Gamma * netCharge.m == GammaQ_vector.m on the reference's 4x4x4 quartz."""
    import largetb_gb300 as T
    q = T.model_quartz(4, 4, 4)
    with gpu.Context() as c:
        c.set_hamiltonian(q.rowptr, q.colidx, q.vals, q.orb2atom, q.natoms)
        c.set_scc(q.g_rowptr, q.g_colidx, q.g_vals, np.zeros(q.natoms))
        V = c.coulomb_shift(golden["netcharge"])
    np.testing.assert_allclose(V, golden["gammaq"], atol=1e-13, rtol=0)


@pytest.mark.parametrize("prec", [0, 1])
def test_scc_matches_oracle(gpu, prec):
    m, o = _pair(2, 2, 2)
    ref = O.scc(o, O.kpe_params(M=200, kT=0.01, n_elec=o.n_elec), tol=1e-6, max_iter=100,
                beta=0.2, history=16)
    assert ref["status"] == 0
    with _ctx(gpu, m, M=200, precision=prec) as c:
        r = c.scc_solve()
    assert abs(r["iters"] - ref["iters"]) <= 1
    assert np.abs(r["q"] - ref["q"]).max() < 1e-6
    assert abs(r["e_band"] - ref["e_band"]) / m.natoms < 1e-7
    assert r["report"]["dq_max"] < 1e-6


def test_scc_with_initial_charges(gpu):
    m, o = _pair(1, 1, 2, seed=3)
    p = O.kpe_params(M=100, kT=0.01, n_elec=o.n_elec)
    ref = O.scc(o, p, tol=1e-6, max_iter=100, beta=0.2, history=16)
    with _ctx(gpu, m, M=100) as c:
        r = c.scc_solve(q_init=ref["q"])
        r0 = c.scc_solve()
    # a warm start at the converged charges needs a few iterations at most;
    # two runs that each stop at max|q_out - q_in| < 1e-6 sit within a few
    # 1e-6 of each other (the residual bounds the step, not the distance to
    # the fixed point), so the warm start is held to 3e-6 of the cold start
    assert r["iters"] <= 4 and r["iters"] < r0["iters"]
    assert r["report"]["dq_max"] < 1e-6
    assert np.abs(r["q"] - r0["q"]).max() < 3e-6


def test_scc_reference_sign_diverges_or_caps(gpu):
    import largetb_gb300 as T
    m, _ = _pair(1, 1, 2, seed=3, gamma_diag=-1.0)
    with _ctx(gpu, m, M=100, scc_max_iter=25) as c:
        with pytest.raises(T.TbError) as e:
            c.scc_solve()
    assert e.value.status in (T.api.TB_ERR_NOT_CONVERGED, T.api.TB_ERR_DIVERGED)


def test_invalid_inputs(gpu):
    import largetb_gb300 as T
    m, _ = _pair(1, 1, 1)
    c = T.Context()
    with pytest.raises(T.TbError) as e:
        c.density()
    assert e.value.status == T.api.TB_ERR_NOT_READY
    bad = m.vals.copy()
    bad[5] = np.nan
    with pytest.raises(T.TbError) as e:
        c.set_hamiltonian(m.rowptr, m.colidx, bad, m.orb2atom, m.natoms)
    assert e.value.status == T.api.TB_ERR_NONFINITE
    o2a = m.orb2atom.copy()
    o2a[4], o2a[5] = 2, 1
    with pytest.raises(T.TbError) as e:
        c.set_hamiltonian(m.rowptr, m.colidx, m.vals, o2a, m.natoms)
    assert e.value.status == T.api.TB_ERR_STRUCTURE
    col = m.colidx.copy()
    col[0], col[1] = col[1], col[0]
    with pytest.raises(T.TbError) as e:
        c.set_hamiltonian(m.rowptr, col, m.vals, m.orb2atom, m.natoms)
    assert e.value.status == T.api.TB_ERR_STRUCTURE
    c.set_model(m)
    c.set_params(n_electrons=3.0 * m.n)  # more electrons than states
    with pytest.raises(T.TbError) as e:
        c.density()
    assert e.value.status == T.api.TB_ERR_BISECTION
    c.close()


def test_asymmetric_input_is_symmetrised(gpu):
    """runKPM symmetrises (H + H^T)/2 (withSP2_deltaH.cpp:1536-1538)."""
    m, o = _pair(1, 1, 2, seed=5)
    vals = m.vals.copy()
    rng = np.random.default_rng(1)
    vals += rng.normal(0, 1e-3, vals.shape)
    H = np.zeros((m.n, m.n))
    for i in range(m.n):
        H[i, m.colidx[m.rowptr[i]:m.rowptr[i + 1]]] = vals[m.rowptr[i]:m.rowptr[i + 1]]
    Hs = 0.5 * (H + H.T)
    o.val[:] = Hs[np.repeat(np.arange(m.n), np.diff(o.rowptr)), o.col]
    ref = O.density(o, O.kpe_params(M=100, kT=0.01, n_elec=o.n_elec))
    with _ctx(gpu, m, M=100) as c:
        c.set_hamiltonian(m.rowptr, m.colidx, vals, m.orb2atom, m.natoms)
        c.set_scc(m.g_rowptr, m.g_colidx, m.g_vals, m.q0)
        r = c.density()
    assert r["report"]["asym_max"] > 1e-4
    assert np.abs(r["q"] - ref["q"]).max() < 1e-9


def test_lower_triangle_only_input_is_completed(gpu):
    m, o = _pair(1, 1, 2, seed=5)
    ref = O.density(o, O.kpe_params(M=100, kT=0.01, n_elec=o.n_elec))
    # keep only j <= i, double the off-diagonal values: (H + H^T)/2 restores H
    rows, cols, vals = [], [], []
    for i in range(m.n):
        for k in range(m.rowptr[i], m.rowptr[i + 1]):
            j = m.colidx[k]
            if j <= i:
                rows.append(i)
                cols.append(j)
                vals.append(m.vals[k] * (1.0 if j == i else 2.0))
    rows = np.array(rows)
    rp = np.zeros(m.n + 1, np.int32)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    with _ctx(gpu, m, M=100) as c:
        c.set_hamiltonian(rp, np.array(cols, np.int32), np.array(vals), m.orb2atom, m.natoms)
        c.set_scc(m.g_rowptr, m.g_colidx, m.g_vals, m.q0)
        r = c.density()
    assert np.abs(r["q"] - ref["q"]).max() < 1e-9


def test_full_size_fp32_vs_fp64_properties(gpu):
    """6x6x6 cristobalite (5184 atoms, 20736 orbitals), M=400: the FP32 form
    against the plain FP64 form on the GPU, plus size-independent checks."""
    import largetb_gb300 as T
    m = T.model_cristobalite(6, 6, 6, sigma_ang=0.05, seed=2002)
    out = {}
    for prec in (0, 1):
        with _ctx(gpu, m, M=400, precision=prec) as c:
            out[prec] = c.density()
    q64, q32 = out[0]["q"], out[1]["q"]
    assert abs(q64.sum() - m.n_electrons) < 1e-6
    assert abs(q32.sum() - m.n_electrons) < 1e-5
    assert np.abs(q32 - q64).max() < 1e-6
    assert abs(out[0]["e_band"] - out[1]["e_band"]) / m.natoms < 1e-7
    # mu_0 = tr I = n exactly; tr X equals the scaled trace of H
    assert abs(out[0]["moments"][0] - m.n) < 1e-9
    assert np.all(out[0]["diagP"] > -1e-6) and np.all(out[0]["diagP"] < 1 + 1e-6)


@pytest.mark.parametrize("kern", [1, 2, 3, 4])
@pytest.mark.parametrize("dims,B", [((2, 2, 2), 0), ((1, 2, 3), 0), ((2, 2, 2), 128), ((1, 1, 3), 256)])
def test_fp32_step_kernels_match_oracle(gpu, kern, dims, B):
    """Each FP32 step kernel (staged, persistent, pipelined with one launch per
    slab, pipelined with one launch per step), forced, with the autotuned and
    with fixed slab widths, against the FP64 oracle."""
    m, o = _pair(*dims, seed=23)
    ref = O.density(o, O.kpe_params(M=160, kT=0.01, n_elec=o.n_elec))
    with _ctx(gpu, m, M=160, precision=gpu.PREC_FP32, fp32_kernel=kern, column_block=B) as c:
        r = c.density()
    rep = r["report"]
    assert rep["step_kernel"] == kern
    if kern != 2 and B:
        assert rep["column_block"] == min(B, -(-m.n // 64) * 64)
    assert np.abs(r["q"] - ref["q"]).max() < 1e-6
    assert abs(r["e_band"] - ref["e_band"]) / m.natoms < 1e-7
    assert abs(r["q"].sum() - m.n_electrons) < 1e-6


def test_pipelined_equals_staged_recurrence(gpu):
    """The pipelined and staged kernels run the same FP32 multiply-add chain
    per block row; only the FP64 order of the row partials differs, so the
    charges agree far below the FP32 tolerance."""
    import largetb_gb300 as T
    m = T.model_cristobalite(3, 3, 3, sigma_ang=0.08, seed=31)
    out = {}
    for kern in (1, 3, 4):
        with _ctx(gpu, m, M=300, precision=gpu.PREC_FP32, fp32_kernel=kern, column_block=512) as c:
            out[kern] = c.density()
    for kern in (3, 4):
        assert np.abs(out[1]["q"] - out[kern]["q"]).max() < 1e-10
        np.testing.assert_allclose(out[1]["moments"], out[kern]["moments"], rtol=0, atol=1e-9 * m.n)
    # the two pipelined modes run identical arithmetic in the same order
    assert np.array_equal(out[3]["moments"], out[4]["moments"])


def test_autotuner_reports_a_kernel(gpu):
    import largetb_gb300 as T
    m = T.model_cristobalite(2, 2, 3, sigma_ang=0.05, seed=5)
    with _ctx(gpu, m, M=60, precision=gpu.PREC_FP32) as c:
        rep = c.density()["report"]
        again = c.density()["report"]
    assert rep["step_kernel"] in (1, 2, 3, 4)
    assert (again["step_kernel"], again["column_block"]) == (rep["step_kernel"], rep["column_block"])


def test_fp32_check_reports_recurrence_error(gpu, cfg1):
    """check_fp32: tb_density reruns 64 identity columns in the plain FP64
    form at the same a, b and reports the largest diagP difference there --
    the FP32 recurrence error alone (same mu and coefficients for both)."""
    m, o, ref = cfg1
    with _ctx(gpu, m, M=200, precision=gpu.PREC_FP32, check_fp32=1) as c:
        r = c.density()
    rep = r["report"]
    assert 0 < rep["fp32_diag_err"] < 1e-6
    assert rep["fp32_check_ms"] > 0
    # the FP32 diagP of those orbitals against the oracle's FP64 ones: same order
    assert np.abs(r["diagP"][:64] - ref["diagP"][:64]).max() < 1e-6
    with _ctx(gpu, m, M=200, precision=gpu.PREC_FP32) as c:
        assert c.density()["report"]["fp32_diag_err"] == 0.0


@pytest.mark.parametrize("prec", [0, 1])
def test_scc_graph_replay_equals_direct_launches(gpu, prec):
    """The SCC iteration replayed from its captured CUDA graph gives the same
    charges, iterations and launch counts as launching every kernel directly;
    changing a parameter invalidates the graph.  The FP32 step kernel and
    slab width are pinned (the per-step launch, captured in the graph): the
    autotuner picks by timing, and another kernel sums the column products
    in another order."""
    m, _ = _pair(2, 2, 2, seed=19)
    pin = dict(fp32_kernel=gpu.FP32_PIPELINED_STEP, column_block=256) if prec == gpu.PREC_FP32 else {}
    out = {}
    for ng in (0, 1):
        with _ctx(gpu, m, M=160, precision=prec, no_graphs=ng, **pin) as c:
            r = c.scc_solve()
            c.set_params(mix_beta=0.3)
            r2 = c.scc_solve()
        out[ng] = (r, r2)
    for i in (0, 1):
        a, b = out[0][i], out[1][i]
        assert a["iters"] == b["iters"]
        np.testing.assert_array_equal(a["q"], b["q"])
        assert a["report"]["kernel_launches"] == b["report"]["kernel_launches"]
        assert a["report"]["step_kernel"] == b["report"]["step_kernel"]
        assert a["report"]["t_moments_ms"] > 0
    assert out[0][0]["iters"] != out[0][1]["iters"] or not np.array_equal(out[0][0]["q"], out[0][1]["q"])


def test_large_cell_properties(gpu):
    """8x8x8 cristobalite (12288 atoms, 49152 orbitals), M = 200, FP32 form
    with the autotuned kernel: size-independent properties -- the electron
    count, 0 <= diagP <= 1, the in-call FP64 check of 64 columns within the
    1e-6 e bar, and the two pipelined launch modes agreeing to round-off."""
    m = gpu.model_cristobalite(8, 8, 8, sigma_ang=0.08, seed=8008)
    with _ctx(gpu, m, M=200, precision=gpu.PREC_FP32, check_fp32=1) as c:
        r = c.density()
    rep = r["report"]
    assert abs(r["q"].sum() - m.n_electrons) < 1e-5
    assert r["diagP"].min() > -1e-6 and r["diagP"].max() < 1 + 1e-6
    assert rep["fp32_diag_err"] < 1e-6
    out = {}
    for kern in (3, 4):
        with _ctx(gpu, m, M=200, precision=gpu.PREC_FP32, fp32_kernel=kern, column_block=1024) as c:
            out[kern] = c.density()
    assert np.array_equal(out[3]["moments"], out[4]["moments"])
    assert np.abs(out[4]["q"] - r["q"]).max() < 1e-9


def test_contexts_with_different_plans_coexist(gpu):
    """Two live contexts whose pipelined plans need different shared memory:
    the later (smaller) plan must not cap the earlier context's launches."""
    big = gpu.model_cristobalite(2, 2, 3, sigma_ang=0.05, seed=41)    # R = 24 groups
    small = gpu.model_cristobalite(1, 1, 1, sigma_ang=0.05, seed=42)  # a different R
    a = _ctx(gpu, big, M=80, precision=gpu.PREC_FP32, fp32_kernel=4, column_block=256)
    ra = a.density()
    b = _ctx(gpu, small, M=80, precision=gpu.PREC_FP32, fp32_kernel=4, column_block=128)
    b.density()
    ra2 = a.density()
    np.testing.assert_array_equal(ra["q"], ra2["q"])
    a.close()
    b.close()


def test_edge_sizes(gpu):
    """Empty and mismatched inputs are refused with a status; a single
    isolated atom (one 4x4 diagonal block, a ragged 4-column slab) gives the
    occupations of its own levels; the smallest and largest expansion orders
    run (M = 2, M = 6000) and M = 6001 is refused."""
    import largetb_gb300 as T
    with T.Context() as c:
        e0 = np.zeros(0, np.int32)
        with pytest.raises(T.TbError) as e:
            c.set_hamiltonian(np.zeros(1, np.int32), e0, np.zeros(0), e0, 0)
        assert e.value.status == T.api.TB_ERR_INVALID_ARG
        rp = np.arange(0, 17, 4, dtype=np.int32)
        ci = np.tile(np.arange(4, dtype=np.int32), 4)
        with pytest.raises(T.TbError) as e:  # 4 orbitals declared as 2 atoms
            c.set_hamiltonian(rp, ci, np.eye(4).ravel(), np.array([0, 0, 1, 1], np.int32), 2)
        assert e.value.status == T.api.TB_ERR_STRUCTURE
    # one isolated atom: levels -0.5 (s) and 0.2 (p x3), 2 electrons fill the s level
    h = np.diag([-0.5, 0.2, 0.2, 0.2]).ravel()
    for prec in (0, 1):
        with T.Context(M=400, kT=0.005, n_electrons=2.0, precision=prec, spectral_pad=0.05) as c:
            c.set_hamiltonian(rp, ci, h, np.zeros(4, np.int32), 1)
            r = c.density()
        np.testing.assert_allclose(r["diagP"], [1, 0, 0, 0], atol=1e-4)
        assert abs(r["q"][0] - 2.0) < 1e-6
    m, o = _pair(1, 1, 1, seed=3)
    for M in (2, 6000):
        with _ctx(gpu, m, M=M, precision=1, kT=0.05) as c:
            r = c.density()
        assert abs(r["q"].sum() - m.n_electrons) < 1e-5
        if M == 6000:
            ref = O.density(o, O.kpe_params(M=M, kT=0.05, n_elec=o.n_elec))
            assert np.abs(r["q"] - ref["q"]).max() < 1e-6
    p = T.params(M=6001)
    h_ = T.api._vp()
    assert T.load().tb_ctx_create(T.api.C.byref(p), T.api.C.byref(h_)) == T.api.TB_ERR_INVALID_ARG
