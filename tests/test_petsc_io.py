"""PETSc MATLAB-dump I/O (CPU) and the GPU path on the reference's own H.m."""
import os

import numpy as np
import pytest

from largetb_gb300 import petsc_io
from oracle import oracle as O


def _golden_csr(g, key):
    r, c, v = g[key + "_r"].astype(np.int64), g[key + "_c"].astype(np.int64), g[key + "_v"]
    return petsc_io.coo_to_csr(r, c, v, tuple(g[key + "_shape"]))


def test_roundtrip(tmp_path, golden):
    rp, ci, va, shape = _golden_csr(golden, "amat")
    p = tmp_path / "Amat.m"
    petsc_io.write_mat(p, rp, ci, va, shape)
    rp2, ci2, va2, shape2 = petsc_io.read_mat(p)
    assert shape2 == shape
    np.testing.assert_array_equal(rp2, rp)
    np.testing.assert_array_equal(ci2, ci)
    np.testing.assert_array_equal(va2, va)
    v = golden["gammaq"]
    petsc_io.write_vec(tmp_path / "v.m", v)
    np.testing.assert_array_equal(petsc_io.read_vec(tmp_path / "v.m"), v)


def test_reference_h_is_what_the_oracle_builds(golden):
    rp, ci, va, shape = _golden_csr(golden, "h444")
    m = O.quartz(4, 4, 4)
    np.testing.assert_array_equal(rp, m.rowptr)
    np.testing.assert_array_equal(ci, m.col)
    np.testing.assert_allclose(va, m.val, atol=1e-14, rtol=0)


@pytest.mark.gpu
def test_gpu_density_on_reference_h(gpu, golden):
    """The reference's own 4x4x4 alpha-quartz Hamiltonian (H.m, 2304 orbitals,
    48 electrons per 9-atom cell) through tb_set_hamiltonian, against the
    oracle on the same CSR."""
    rp, ci, va, shape = _golden_csr(golden, "h444")
    natoms = shape[0] // 4
    n_e = 64 * 48.0  # Nelectrons of withSP2_deltaH.cpp:1766 for 4x4x4
    o = O.model_from_csr(rp, ci, va, natoms)
    ref = O.density(o, O.kpe_params(M=200, kT=0.01, n_elec=n_e))
    o2a = np.repeat(np.arange(natoms, dtype=np.int32), 4)
    for prec, tol in ((gpu.PREC_FP64, 1e-9), (gpu.PREC_FP32, 1e-6)):
        with gpu.Context(M=200, precision=prec, n_electrons=n_e) as c:
            c.set_hamiltonian(rp, ci, va, o2a, natoms)
            r = c.density()
        assert np.abs(r["q"] - ref["q"]).max() < tol
        assert abs(r["e_band"] - ref["e_band"]) / natoms < 1e-7
