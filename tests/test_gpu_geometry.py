"""H, Gamma and q0 built on the GPU (tb_set_geometry) against the host-built
model: same density and SCC results (FP64: to round-off)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOHR_PER_ANG = 1.88973


def test_device_built_model_matches_host_model(gpu):
    for dims, sig, seed in [((2, 2, 2), 0.05, 1001), ((2, 1, 3), 0.12, 5)]:
        m = gpu.model_cristobalite(*dims, sigma_ang=sig, seed=seed)
        box = np.array(dims, float) * 7.16 * BOHR_PER_ANG
        with gpu.Context(M=150) as a, gpu.Context(M=150) as b:
            a.set_model(m)
            b.set_geometry(m.xyz, m.species, box, rcut_bohr=4.0, gamma_diag=1.0)
            ra, rb = a.density(), b.density()
            assert np.abs(ra["q"] - rb["q"]).max() < 1e-11
            assert abs(ra["e_band"] - rb["e_band"]) < 1e-9
            sa, sb = a.scc_solve(), b.scc_solve()
            assert sa["iters"] == sb["iters"]
            assert np.abs(sa["q"] - sb["q"]).max() < 1e-9


def test_geometry_validation(gpu):
    m = gpu.model_cristobalite(1, 1, 1, sigma_ang=0.0, seed=0)
    with gpu.Context() as c:
        with pytest.raises(gpu.TbError):
            c.set_geometry(m.xyz, m.species, [5.0, 5.0, 5.0], rcut_bohr=4.0)  # box < 2 rcut
        sp = m.species.copy()
        sp[0] = 6
        with pytest.raises(gpu.TbError):
            c.set_geometry(m.xyz, sp, [13.53, 13.53, 13.53], rcut_bohr=4.0)
