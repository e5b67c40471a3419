import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) CUDA device")


def _has_gpu():
    try:
        import largetb_gb300 as T
        c = T.Context()
        c.close()
        return True
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not _has_gpu():
        pytest.fail("no usable sm_103 device or libtb_gb300.so failed to load")
    import largetb_gb300 as T
    return T


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_dumps.npz"))


def dense_coo(g, key):
    import numpy as np
    A = np.zeros(tuple(g[key + "_shape"]))
    A[g[key + "_r"], g[key + "_c"]] = g[key + "_v"]
    return A


def reference_dos(g):
    """The reference's DOS of Htotal_scc (dosfile.txt, runKPM of
    withSP2_deltaH.cpp:1579-1718) turned back into its moments.

    runKPM prints rho(x_q) = [g_0 mu_0 + 2 sum_{k>=1} g_k mu_k cos(k theta_q)]
    / (pi sin theta_q) at theta_q = pi (q + 1/2) / (2 N), q < 2 N, with N = 1000
    Jackson-damped moments mu_k = sum_r r^T T_k(X) r over its Gaussian vectors
    r and E_q = a cos theta_q + b.  The cosine sums are a discrete cosine
    transform, so g_k mu_k = (1/2N) sum_q pi sin theta_q rho_q cos(k theta_q)
    exactly (up to the 6-decimal print).  Returns (H symmetrised as runKPM
    does, a, b, mu_ref, n_vectors)."""
    import numpy as np
    import scipy.sparse as sp
    from oracle import oracle as O
    n = int(g["hscc_shape"][0])
    H = sp.csr_matrix((g["hscc_v"], (g["hscc_r"], g["hscc_c"])), shape=(n, n))
    H = ((H + H.T) / 2).tocsr()  # MatTranspose + MatAXPY, withSP2_deltaH.cpp:1536-1538
    H.sort_indices()
    E, rho = g["dosfile"][:, 0], g["dosfile"][:, 1]
    nt = len(E)
    th = np.pi * (np.arange(nt) + 0.5) / nt
    a = (E[0] - E[-1]) / (2 * np.cos(th[0]))
    b = (E[0] + E[-1]) / 2
    f = np.pi * np.sin(th) * rho
    k = np.arange(nt // 2)
    gmu = (np.cos(np.outer(k, th)) @ f) / nt
    mu = gmu / O.jackson(nt // 2)
    return H, a, b, mu, mu[0] / n


def moment_z(mu_ref, nvec, tr, n, K):
    """z-scores of the reference's stochastic moments against exact traces
    tr[0..2K]: Var(sum_r r^T A r) = 2 nvec ||A||_F^2 for Gaussian r and
    ||T_k||_F^2 = (tr T_2k + n) / 2."""
    import numpy as np
    fro2 = (np.asarray(tr[0:2 * K:2]) + n) / 2
    sig = np.sqrt(2 * nvec * fro2) / nvec
    return (mu_ref[:K] / nvec - np.asarray(tr[:K])) / sig
