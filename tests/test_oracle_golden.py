"""The FP64 CPU oracle against the reference's own dumps and against exact
linear algebra (CPU only)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import dense_coo


def _gamma_dense(m):
    G = np.zeros((m.natoms, m.natoms))
    for a in range(m.natoms):
        s, e = m.g_rowptr[a], m.g_rowptr[a + 1]
        G[a, m.g_col[s:e]] = m.g_val[s:e]
    return G


def test_amat_1x1x1_quartz(golden):
    m = O.quartz(1, 1, 1)
    A = dense_coo(golden, "amat")
    assert m.rowptr[-1] == len(golden["amat_v"])  # same stored entries (explicit zeros kept)
    np.testing.assert_allclose(m.dense_h(), A, atol=1e-14, rtol=0)


def test_h_4x4x4_quartz(golden):
    m = O.quartz(4, 4, 4)
    A = dense_coo(golden, "h444")
    assert m.rowptr[-1] == len(golden["h444_v"])
    np.testing.assert_allclose(m.dense_h(), A, atol=1e-14, rtol=0)


def test_gamma_and_orbital_map(golden):
    m = O.quartz(4, 4, 4)
    np.testing.assert_allclose(_gamma_dense(m), dense_coo(golden, "gamma"), atol=1e-14, rtol=0)
    o2a = dense_coo(golden, "o2a")
    mine = (np.arange(m.natoms)[:, None] == m.orb2atom[None, :]).astype(float)
    np.testing.assert_array_equal(o2a, mine)


def test_coulomb_shift_known_answer(golden):
    """netCharge.m -> GammaQ_vector.m -> deltaH.m of one reference SCC step."""
    m = O.quartz(4, 4, 4)
    gq = O.gamma_mult(m, golden["netcharge"])
    np.testing.assert_allclose(gq, golden["gammaq"], atol=1e-13, rtol=0)
    dh = dense_coo(golden, "dh")
    np.testing.assert_array_equal(np.diag(dh), np.repeat(golden["gammaq"], 4))
    assert np.abs(dh - np.diag(np.diag(dh))).max() == 0.0


def test_jackson_against_gnsfile(golden):
    g = O.jackson(1000)
    np.testing.assert_allclose(g, golden["gns_col1"], atol=6e-7, rtol=0)  # 6-digit print


def test_autocorr_kernel_definition():
    M = 50
    g = O.kernel_autocorr(M)
    al = np.pi / (M + 2)
    u = np.sin((np.arange(M) + 1) * al) / np.sin(al)
    u /= np.linalg.norm(u)
    ref = np.array([sum(u[i] * u[m + i] for i in range(M - m - 1)) for m in range(M)])
    np.testing.assert_allclose(g, ref, atol=1e-15)


@pytest.mark.parametrize("mu", [-0.7, 0.0, 0.31])
def test_fermi_coeffs_reduce_to_step(mu):
    M = 64
    step = O.step_coeffs(M, mu)
    cold = O.fermi_coeffs(M, mu, beta_x=1e5)
    np.testing.assert_allclose(cold, step, atol=2e-4)
    # a smooth Fermi function: quadrature converged (doubling nodes changes nothing)
    c1 = O.fermi_coeffs(M, mu, 200.0, nq=4096)
    c2 = O.fermi_coeffs(M, mu, 200.0, nq=8192)
    np.testing.assert_allclose(c1, c2, atol=1e-14)


def _small():
    return O.cristobalite(1, 1, 2, sigma_ang=0.05, seed=7)


def test_exact_moments_against_eigendecomposition():
    m = _small()
    lo, hi = O.gershgorin(m)
    a, b = (hi - lo) / 2, (hi + lo) / 2
    M = 60
    d = O.exact_moments(m, a, b, M + 1)
    w, U = np.linalg.eigh(m.dense_h())
    x = (w - b) / a
    T = np.cos(np.outer(np.arange(M + 1), np.arccos(np.clip(x, -1, 1))))
    np.testing.assert_allclose(d, (U ** 2 @ T.T).T, atol=1e-11)
    # column-range restatement gives the same columns
    d2 = O.exact_moments_cols(m, a, b, M + 1, 40, 100)
    np.testing.assert_allclose(d2[:, 40:100], d[:, 40:100], atol=0, rtol=0)


def test_density_against_eigendecomposition():
    m = _small()
    p = O.kpe_params(M=300, kT=0.01, n_elec=m.n_elec)
    r = O.density(m, p)
    assert abs(r["n_elec_found"] - m.n_elec) < 1e-8
    assert abs(r["q"].sum() - m.n_elec) < 1e-8
    w, U = np.linalg.eigh(m.dense_h())
    # P = sum_n c_n g_n T_n(X) evaluated on the eigenvalues
    g = O.jackson(300)
    c = O.fermi_coeffs(300, r["mu_x"], r["a"] / 0.01)
    x = (w - r["b"]) / r["a"]
    f = (c * g) @ np.cos(np.outer(np.arange(300), np.arccos(x)))
    np.testing.assert_allclose(r["diagP"], U ** 2 @ f, atol=1e-10)
    assert abs(r["e_band"] - 2 * (f * w).sum()) < 1e-9


def test_step_function_density():
    m = _small()
    r = O.density(m, O.kpe_params(M=200, kT=0.0, n_elec=m.n_elec))
    assert abs(r["n_elec_found"] - m.n_elec) < 1e-6


def test_bisection_failure_is_reported():
    m = _small()
    with pytest.raises(O.OracleError):
        O.density(m, O.kpe_params(M=50, kT=0.01, n_elec=2.5 * m.n))


def test_scc_converges_with_physical_sign_and_not_with_reference_sign():
    """Gamma_aa = -U (withSP2_deltaH.cpp:876-899) drives charge runaway; +U converges."""
    m = _small()
    p = O.kpe_params(M=120, kT=0.01, n_elec=m.n_elec)
    r = O.scc(m, p, tol=1e-6, max_iter=60, beta=0.2, history=8)
    assert r["status"] == 0 and r["iters"] < 40
    assert abs(r["q"].sum() - m.n_elec) < 1e-7
    bad = O.cristobalite(1, 1, 2, sigma_ang=0.05, seed=7, gamma_diag=-1.0)
    rb = O.scc(bad, p, tol=1e-6, max_iter=30, beta=0.2, history=8)
    assert rb["status"] != 0


def test_anderson_without_history_is_linear_mixing():
    m = _small()
    p = O.kpe_params(M=120, kT=0.01, n_elec=m.n_elec)
    r = O.scc(m, p, tol=1e-6, max_iter=3, beta=0.1, history=0)
    assert r["iters"] == 3


def test_product_builder_matches_oracle():
    import largetb_gb300 as T
    for nx, ny, nz, sig, seed in [(1, 1, 2, 0.05, 7), (2, 2, 2, 0.05, 1001), (2, 1, 3, 0.12, 5)]:
        a = T.model_cristobalite(nx, ny, nz, sigma_ang=sig, seed=seed)
        b = O.cristobalite(nx, ny, nz, sigma_ang=sig, seed=seed)
        np.testing.assert_array_equal(a.rowptr, b.rowptr)
        np.testing.assert_array_equal(a.colidx, b.col)
        np.testing.assert_allclose(a.vals, b.val, atol=1e-14, rtol=0)
        np.testing.assert_array_equal(a.g_colidx, b.g_col)
        np.testing.assert_allclose(a.g_vals, b.g_val, atol=1e-14, rtol=0)
        np.testing.assert_allclose(a.xyz, b.xyz, atol=1e-12, rtol=0)
    q = T.model_quartz(2, 2, 1)
    oq = O.quartz(2, 2, 1)
    np.testing.assert_allclose(q.vals, oq.val, atol=1e-14, rtol=0)


def test_moments_pinned_by_reference_dos(golden):
    """Statistical pin of the KPE recurrence on a reference matrix: the
    oracle's exact traces tr T_k((H - b)/a) of Htotal_scc, at the reference's
    own a, b, against the moments behind the reference's 20-vector DOS
    (dosfile.txt).  A different matrix (H.m) scores mean z^2 in the
    thousands."""
    from tests.conftest import moment_z, reference_dos
    H, a, b, mu, nvec = reference_dos(golden)
    n = H.shape[0]
    assert abs(nvec - 20) < 1.5  # runKPM's nRandoms
    m = O.model_from_csr(H.indptr, H.indices, H.data, n // 4)
    K = 120
    tr = O.exact_moments(m, a, b, 2 * K + 1).sum(1)
    assert abs(tr[0] - n) < 1e-9
    z = moment_z(mu, nvec, tr, n, K)[1:]
    assert np.abs(z).max() < 5 and np.mean(z ** 2) < 2


def test_headline_oracle_fixture_is_this_model():
    """The committed FP64-oracle SCC of the 6x6x6 cell (tests/golden/
    make_scc_oracle.py) was computed on the Hamiltonian the oracle builds
    today: same size, pattern and value sums; its run converged (24
    iterations to 1e-6 e, residual history falling to 1e-8 e) and holds the
    electron count."""
    import os
    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scc_oracle_6x6x6.npz"))
    m = O.cristobalite(6, 6, 6, sigma_ang=float(fx["sigma_ang"]), seed=int(fx["seed"]))
    ms = fx["model_sums"]
    assert m.n == int(ms[0]) and m.rowptr[-1] == int(ms[1])
    np.testing.assert_allclose([np.sum(m.val), np.sum(m.val * m.val), np.sum(np.abs(m.val)), np.sum(m.xyz)],
                               ms[2:], rtol=1e-12)
    it = int(fx["iters"])
    assert fx["dq_hist"][it - 1] < 1e-6 <= fx["dq_hist"][it - 2]
    assert fx["dq_hist"][-1] < float(fx["tight_tol"])
    assert abs(fx["q"].sum() - m.n_elec) < 1e-6
    assert np.abs(fx["q"] - fx["q_tight"]).max() < 1e-6


def _dos_mu_restated(dos, n_elec, n):
    """runKPM's chemical potential and refined interval from a DOS on the
    Chebyshev nodes x_i = cos(pi (i + 1/2) / npts) (withSP2_deltaH.cpp:
    1663-1703), restated in numpy: trapezoid area from the bottom node up,
    the first node where it reaches N_e / 2n of the total; the interval where
    DOS / n >= 0.001 first holds from either end (-10, 10 if never)."""
    npts = len(dos)
    x = np.cos(np.pi * (np.arange(npts) + 0.5) / npts)
    seg = (x[:-1] - x[1:]) * (dos[1:] + dos[:-1]) / 2  # segment i-1..i, for i = npts-1 .. 1
    area = n_elec * seg.sum() / (2.0 * n)
    cum = np.cumsum(seg[::-1])  # from the bottom node upwards
    hit = np.nonzero(cum >= area)[0]
    mi = (npts - 1 - hit[0]) if len(hit) else 0
    above = np.nonzero(dos / n >= 0.001)[0]
    lo_i = above.max() if len(above) else None
    hi_i = above.min() if len(above) else None
    return mi, lo_i, hi_i, x


@pytest.mark.parametrize("gap", [0.0, 0.4])
def test_dos_mu_matches_a_restatement_of_the_area_rule(gap):
    """The oracle's mu and interval (orc_dos_mu) against an independent
    numpy restatement of runKPM's rule, on a two-band DOS (valence and
    conduction Gaussians, with and without a gap) evaluated on the nodes."""
    npts, n, n_elec = 2000, 768, 1024.0
    a, b = 1.3, -0.4
    x = np.cos(np.pi * (np.arange(npts) + 0.5) / npts)
    E = a * x + b
    dos = (2 * n / 3) * np.exp(-((x + 0.35 + gap / 2) / 0.12) ** 2) + (n / 3) * np.exp(-((x - 0.35 - gap / 2) / 0.1) ** 2)
    r = O.dos_mu(E, dos, n_elec, n)
    mi, lo_i, hi_i, _ = _dos_mu_restated(dos, n_elec, n)
    assert r["mu_index"] == mi and r["mu"] == E[mi]
    assert abs(r["a"] - (E[hi_i] - E[lo_i]) / 2) < 1e-12
    assert abs(r["b"] - (E[hi_i] + E[lo_i]) / 2) < 1e-12
    # mu sits where the valence band's share of the area is exhausted
    assert E[mi] < b + a * (0.35 + gap / 2)
