"""The headline cell against the FP64 oracle's converged SCC.

6x6x6 beta-cristobalite (5184 atoms, 20736 orbitals, sigma 0.05 A, seed
2002), M = 400, kT = 0.01 Ha, exact trace, |dq| < 1e-6 e.  The oracle's SCC
(orc_density + orc_anderson in orc_scc's order, Anderson 16 / 0.2 from q0)
ran to convergence on the CPU and is committed as a fixture
(tests/golden/make_scc_oracle.py): its charges, band energy and iteration
count where the residual first fell below 1e-6 e, and the same run carried
on to 1e-8 e (the fixed point itself).

  - The plain FP64 GPU form runs the same SCC from q0: iterations within 1,
    charges within 1e-6 e, band energy within 1e-7 Ha/atom of the oracle's.
  - The FP32 form from q0 with the oracle's mixer: iterations within 1,
    charges within 1e-6 e and band energy within 1e-7 Ha/atom of the
    oracle's fixed point.
  - The FP32 form from the learned start (another starting point and mixer)
    lands on the same fixed point: charges within 1e-6 e and band energy
    within 1e-7 Ha/atom of the oracle's fixed point.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scc_oracle_6x6x6.npz")


@pytest.fixture(scope="module")
def cell(gpu):
    if not os.path.exists(FIX):
        pytest.fail("the 6x6x6 FP64-oracle SCC fixture is missing")
    fx = np.load(FIX)
    m = gpu.model_cristobalite(6, 6, 6, sigma_ang=float(fx["sigma_ang"]), seed=int(fx["seed"]))
    # the same Hamiltonian as the oracle's (fingerprints of the fixture's model)
    ms = fx["model_sums"]
    assert m.n == int(ms[0]) and m.rowptr[-1] == int(ms[1])
    assert abs(float(np.sum(m.vals)) - ms[2]) < 1e-9 * abs(ms[2])
    assert abs(float(np.sum(np.abs(m.vals))) - ms[4]) < 1e-9 * ms[4]
    return m, fx


def test_plain_fp64_matches_oracle_scc(gpu, cell):
    m, fx = cell
    with gpu.Context(M=int(fx["M"]), kT=float(fx["kT"]), precision=gpu.PREC_FP64, mix_beta=0.2,
                     mix_history=16, scc_tol=1e-6, scc_max_iter=60) as c:
        c.set_model(m)
        r = c.scc_solve()
    assert abs(r["iters"] - int(fx["iters"])) <= 1, (r["iters"], int(fx["iters"]))
    assert np.abs(r["q"] - fx["q"]).max() < 1e-6
    assert abs(r["e_band"] - float(fx["e_band"])) / m.natoms < 1e-7


def test_fp32_from_q0_matches_oracle_scc(gpu, cell):
    """The FP32 form from the oracle's own start and mixer (q0, Anderson
    16 / 0.2): iteration count within 1 of the oracle's, and the charges and
    band energy of its stopping point within 1e-6 e and 1e-7 Ha/atom of the
    oracle's fixed point."""
    m, fx = cell
    with gpu.Context(M=int(fx["M"]), kT=float(fx["kT"]), precision=gpu.PREC_FP32, mix_beta=0.2,
                     mix_history=16, scc_tol=1e-6, scc_max_iter=60) as c:
        c.set_model(m)
        r = c.scc_solve()
    assert abs(r["iters"] - int(fx["iters"])) <= 1, (r["iters"], int(fx["iters"]))
    assert np.abs(r["q"] - fx["q_tight"]).max() < 1e-6
    assert abs(r["e_band"] - float(fx["e_band_tight"])) / m.natoms < 1e-7


def test_fp32_learned_start_matches_oracle_fixed_point(gpu, cell):
    from largetb_gb300 import learned
    m, fx = cell
    mlp = learned.load(device=0)
    q_init = learned.warm_start(mlp, m, learned.cell_box((6, 6, 6)))
    with gpu.Context(M=int(fx["M"]), kT=float(fx["kT"]), precision=gpu.PREC_FP32,
                     mix_beta=learned.MIX_BETA, mix_history=16, scc_tol=1e-6, scc_max_iter=60) as c:
        c.set_model(m)
        r = c.scc_solve(q_init=q_init)
    assert np.abs(r["q"] - fx["q_tight"]).max() < 1e-6
    assert abs(r["e_band"] - float(fx["e_band_tight"])) / m.natoms < 1e-7
