"""Stochastic-trace density (tb_density_stochastic) against the FP64 oracle.

The reference's default path: runKPM's stochastic DOS, the chemical
potential from its integrated area and the interval refined from its
support (withSP2_deltaH.cpp:1579-1703), then computeDiagonalElements'
random-vector ratio estimator (1296-1399).  The GPU and the oracle draw the
same counter-based Gaussian probes, so they agree to FP64 round-off; against
the exact trace at the same mu and interval the estimator's error has the
variance the Gaussian probes predict, var_i = ((P^2)_ii - P_ii^2) / N.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(cells=(2, 2, 2), seed=1001):
    import largetb_gb300 as T
    return (T.model_cristobalite(*cells, sigma_ang=0.05, seed=seed),
            O.cristobalite(*cells, sigma_ang=0.05, seed=seed))


@pytest.mark.parametrize("kT", [0.01, 0.0])
def test_stochastic_density_matches_oracle(gpu, kT):
    m, o = _pair()
    M, nr, seed, nd, npts = 120, 16, 77, 200, 400
    ref = O.density_stochastic(o, O.kpe_params(M=M, kT=kT, n_elec=o.n_elec), n_random=nr, seed=seed,
                               dos_moments=nd, dos_points=npts)
    with gpu.Context(M=M, kT=kT, precision=gpu.PREC_FP64) as c:
        c.set_model(m)
        r = c.density_stochastic(n_probes=nr, seed=seed, dos_moments=nd, dos_points=npts)
    rep = r["report"]
    assert abs(rep["a"] - ref["a"]) < 1e-12 and abs(rep["b"] - ref["b"]) < 1e-12
    assert abs(r["mu"] - ref["mu"]) < 1e-12
    np.testing.assert_allclose(r["diagP"], ref["diagP"], atol=1e-10, rtol=0)
    np.testing.assert_allclose(r["q"], ref["q"], atol=1e-9, rtol=0)


def _dense_density(o, a, b, mu_x, M, kT):
    """P = sum_{k<M} c_k g_k T_k(X), X = (H - b)/a, dense (n = 768)."""
    H = sp.csr_matrix((o.val, o.col, o.rowptr), shape=(o.n, o.n)).toarray()
    X = (H - b * np.eye(o.n)) / a
    g = O.jackson(M)
    g[0] = 1.0
    c = O.fermi_coeffs(M, mu_x, a / kT) if kT > 0 else O.step_coeffs(M, mu_x)
    w = c * g
    T0, T1 = np.eye(o.n), X.copy()
    P = w[0] * T0 + w[1] * T1
    for k in range(2, M):
        T0, T1 = T1, 2 * X @ T1 - T0
        P += w[k] * T1
    return P


def test_stochastic_density_error_follows_probe_statistics(gpu):
    """z-scores of the GPU estimator against the exact trace at the same mu
    and interval: mean z^2 near 1 and no outliers, for 64 and 256 probes;
    the RMS error falls as 1/sqrt(N)."""
    m, o = _pair()
    M, kT = 120, 0.01
    rms = []
    for nr in (64, 256):
        with gpu.Context(M=M, kT=kT, precision=gpu.PREC_FP64) as c:
            c.set_model(m)
            r = c.density_stochastic(n_probes=nr, seed=5, dos_moments=200, dos_points=400)
        rep = r["report"]
        a, b = rep["a"], rep["b"]
        P = _dense_density(o, a, b, (r["mu"] - b) / a, M, kT)
        ex = np.diag(P)
        var = (np.einsum("ij,ij->i", P, P) - ex ** 2) / nr
        z = (r["diagP"] - ex) / np.sqrt(var)
        assert 0.5 < np.mean(z ** 2) < 2.0, (nr, np.mean(z ** 2))
        assert np.abs(z).max() < 6.0, (nr, np.abs(z).max())
        rms.append(np.sqrt(np.mean((r["diagP"] - ex) ** 2)))
    assert 1.4 < rms[0] / rms[1] < 2.8, rms


def test_stochastic_mu_in_the_gap(gpu):
    """SiO2 has a gap: the DOS-area chemical potential (runKPM's rule, on
    1000 moments and 2000 nodes) lands between the highest occupied and the
    lowest empty eigenvalue of H (dense eigendecomposition), up to a few DOS
    grid spacings -- near the top of the valence band, where the area
    reaches N_e/2n.  With the reference's step coefficients (kT = 0) the
    stochastic charges then hold the electron count to 1 % (the Jackson
    broadening at M = 200 reaches the top valence states: 0.55 % here)."""
    m, o = _pair()
    with gpu.Context(M=200, kT=0.0, precision=gpu.PREC_FP64) as c:
        c.set_model(m)
        r = c.density_stochastic(n_probes=128, seed=9, dos_moments=1000, dos_points=2000)
    H = sp.csr_matrix((o.val, o.col, o.rowptr), shape=(o.n, o.n)).toarray()
    ev = np.linalg.eigvalsh((H + H.T) / 2)
    nocc = int(round(o.n_elec / 2))
    spacing = np.pi * r["report"]["a"] / 2000
    assert ev[nocc - 1] - 3 * spacing <= r["mu"] <= ev[nocc] + 3 * spacing
    assert abs(r["q"].sum() - m.n_electrons) < 0.01 * m.n_electrons
