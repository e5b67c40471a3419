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
