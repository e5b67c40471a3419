"""Stochastic KPM density of states (tb_kpm_dos) against the oracle's
restatement of runKPM's DOS (withSP2_deltaH.cpp:1579-1648), same seeded
probe vectors: FP64 both, agreement to round-off."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_kpm_dos_matches_oracle(gpu):
    m = gpu.model_cristobalite(2, 2, 2, sigma_ang=0.05, seed=1001)
    o = O.cristobalite(2, 2, 2, sigma_ang=0.05, seed=1001)
    with gpu.Context() as c:
        c.set_model(m)
        r = c.kpm_dos(n_moments=300, n_random=10, seed=77, npts=600)
    a, b = r["report"]["a"], r["report"]["b"]
    lo, hi = O.gershgorin(o)
    assert abs(a - (hi - lo) / 2) < 1e-12 and abs(b - (hi + lo) / 2) < 1e-12
    mom, e, dos = O.kpm_dos(o, a, b, nmom=300, n_random=10, seed=77, npts=600)
    np.testing.assert_allclose(r["moments"], mom, atol=1e-9 * 10 * m.n, rtol=0)
    np.testing.assert_allclose(r["energies"], e, atol=1e-12, rtol=0)
    np.testing.assert_allclose(r["dos"], dos, atol=1e-8 * np.abs(dos).max(), rtol=0)


def test_stochastic_paths_repeat_bitwise(gpu):
    """The same probes give the same moments, DOS, mu and charges from run
    to run: the per-step probe dots are summed in a fixed order."""
    m = gpu.model_cristobalite(2, 2, 2, sigma_ang=0.05, seed=1001)
    with gpu.Context(M=120, kT=0.01, precision=gpu.PREC_FP64) as c:
        c.set_model(m)
        d1 = c.kpm_dos(n_moments=300, n_random=64, seed=5, npts=600)
        d2 = c.kpm_dos(n_moments=300, n_random=64, seed=5, npts=600)
        s1 = c.density_stochastic(n_probes=64, seed=9, dos_moments=300, dos_points=600)
        s2 = c.density_stochastic(n_probes=64, seed=9, dos_moments=300, dos_points=600)
    np.testing.assert_array_equal(d1["moments"], d2["moments"])
    np.testing.assert_array_equal(d1["dos"], d2["dos"])
    assert s1["mu"] == s2["mu"]
    np.testing.assert_array_equal(s1["q"], s2["q"])


def test_kpm_dos_statistics(gpu):
    """The stochastic trace estimates tr T_k(X): mu_0 / n_random ~ n and the
    integrated DOS ~ n (up to sampling noise)."""
    m = gpu.model_cristobalite(2, 2, 2, sigma_ang=0.05, seed=1001)
    with gpu.Context(M=200) as c:
        c.set_model(m)
        r = c.kpm_dos(n_moments=200, n_random=64, seed=5, npts=400)
        ex = c.density()
    mu0 = r["moments"][0] / 64
    assert abs(mu0 - m.n) < 5 * np.sqrt(2.0 * m.n / 64)
    x = (r["energies"] - r["report"]["b"]) / r["report"]["a"]
    area = np.trapezoid(r["dos"][::-1], x[::-1])
    assert abs(area / 64 - m.n) / m.n < 0.05
    # first moments against the exact trace (same scaling: pad 0, no shift)
    assert abs(r["moments"][1] / 64 - ex["moments"][1]) < 5 * np.sqrt(2.0 * m.n / 64)


def _reference_hscc(golden):
    """Htotal_scc.m as the reference dumped it (not symmetrised: the C-ABI
    symmetrises like runKPM), as sorted CSR."""
    import scipy.sparse as sp
    n = int(golden["hscc_shape"][0])
    H = sp.csr_matrix((golden["hscc_v"], (golden["hscc_r"], golden["hscc_c"])), shape=(n, n))
    H.sort_indices()
    return H, n


@pytest.mark.parametrize("prec", [0, 1])
def test_moments_pinned_by_reference_dos(gpu, golden, prec):
    """The exact traces of the GPU path (plain FP64 and the FP32 form) on the
    reference's own Htotal_scc, scaled with the reference's refined a, b
    (tb_params.bounds_lo/hi), against the moments behind the reference's
    20-vector DOS (dosfile.txt): sampling noise only (|z| < 5, mean z^2 < 2)."""
    from tests.conftest import moment_z, reference_dos
    Hs, a, b, mu, nvec = reference_dos(golden)
    H, n = _reference_hscc(golden)
    o2a = np.arange(n, dtype=np.int32) // 4
    M, K = 800, 400
    with gpu.Context(M=M, precision=prec, n_electrons=float(n), bounds_lo=b - a, bounds_hi=b + a) as c:
        c.set_hamiltonian(H.indptr.astype(np.int32), H.indices.astype(np.int32), H.data, o2a, n // 4)
        r = c.density()
    rep = r["report"]
    assert abs(rep["a"] - a) < 1e-12 * a and abs(rep["b"] - b) < 1e-12 * a
    tr = r["moments"]
    assert abs(tr[0] - n) < 1e-6
    z = moment_z(mu, nvec, tr, n, K)[1:]
    assert np.abs(z).max() < 5 and np.mean(z ** 2) < 2


def test_dos_reproduces_reference_dosfile(gpu, golden):
    """tb_kpm_dos with runKPM's settings (1000 Jackson moments, 20 Gaussian
    vectors, 2000 nodes) and the reference's a, b on Htotal_scc: the energy
    grid equals dosfile.txt's to its print precision, and the DOS moments of
    two independent 20-vector estimates agree within their joint noise."""
    from tests.conftest import moment_z, reference_dos
    Hs, a, b, mu, nvec = reference_dos(golden)
    H, n = _reference_hscc(golden)
    o2a = np.arange(n, dtype=np.int32) // 4
    E = golden["dosfile"][:, 0]
    with gpu.Context(M=800, n_electrons=float(n), bounds_lo=b - a, bounds_hi=b + a) as c:
        c.set_hamiltonian(H.indptr.astype(np.int32), H.indices.astype(np.int32), H.data, o2a, n // 4)
        d = c.kpm_dos(n_moments=1000, n_random=20, seed=2024, npts=2000)
        ex = c.density()["moments"]
    assert np.abs(d["energies"] - E).max() < 2e-6
    K = 400
    z_ref = moment_z(mu, nvec, ex, n, K)[1:]
    z_gpu = moment_z(d["moments"], 20.0, ex, n, K)[1:]
    zd = (z_ref - z_gpu) / np.sqrt(2.0)
    assert np.abs(zd).max() < 5 and np.mean(zd ** 2) < 2
