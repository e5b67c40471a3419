"""Python host mirror of the C-ABI in include/largetb.h.

The reference's operator surface for this path is a set of PETSc routines on
global state (withSP2_deltaH.cpp): GershGorinParallel (144), runKPM (1528),
computeDensityMatrix (1401), constructdeltaH (1414) and the SCC loop of main
(1820-1840), all returning a PetscErrorCode.  ``Context`` exposes the same
operations as methods on an explicit context; a non-zero status becomes a
``TbError`` carrying the code and ``tb_last_error``.

The CUDA library is loaded from the in-tree build (``largetb_gb300/_build``);
if it is missing or no sm_103 GPU is present the calls fail loudly -- there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

TB_OK = 0
TB_ERR_INVALID_ARG = 1
TB_ERR_STRUCTURE = 2
TB_ERR_NONFINITE = 3
TB_ERR_NOT_READY = 4
TB_ERR_SPECTRUM = 5
TB_ERR_BISECTION = 6
TB_ERR_NOT_CONVERGED = 7
TB_ERR_DIVERGED = 8
TB_ERR_CUDA = 9
TB_ERR_NO_DEVICE = 10
TB_ERR_OUT_OF_MEMORY = 11
TB_ERR_UNSUPPORTED = 12
TB_ERR_TIMEOUT = 13

PREC_FP64 = 0
PREC_FP32 = 1
KERNEL_JACKSON = 0
KERNEL_AUTOCORR = 1
KERNEL_NONE = 2
FP32_AUTO = 0
FP32_STAGED = 1
FP32_PERSISTENT = 2
FP32_PIPELINED = 3
FP32_PIPELINED_STEP = 4
MODE_KPE = 0
MODE_SP2 = 1


class TbParams(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("M", C.c_int32),
        ("kernel", C.c_int32),
        ("precision", C.c_int32),
        ("kT", C.c_double),
        ("n_electrons", C.c_double),
        ("column_block", C.c_int32),
        ("device", C.c_int32),
        ("spectral_pad", C.c_double),
        ("mu_tol", C.c_double),
        ("scc_tol", C.c_double),
        ("scc_max_iter", C.c_int32),
        ("mix_history", C.c_int32),
        ("mix_beta", C.c_double),
        ("sp2_drop_tol", C.c_double),
        ("sp2_max_iter", C.c_int32),
        ("fp32_kernel", C.c_int32),
        ("sp2_idem_tol", C.c_double),
        ("bounds_lo", C.c_double),
        ("bounds_hi", C.c_double),
        ("mode", C.c_int32),
        ("check_fp32", C.c_int32),
        ("no_graphs", C.c_int32),
        ("fp64_small", C.c_int32),
        ("reserved", C.c_double * 2),
    ]


class TbReport(C.Structure):
    _fields_ = [
        ("lmin", C.c_double),
        ("lmax", C.c_double),
        ("a", C.c_double),
        ("b", C.c_double),
        ("mu", C.c_double),
        ("n_electrons_found", C.c_double),
        ("e_band", C.c_double),
        ("dq_max", C.c_double),
        ("scc_iters", C.c_int32),
        ("bisect_rounds", C.c_int32),
        ("column_block", C.c_int32),
        ("precision", C.c_int32),
        ("t_total_ms", C.c_double),
        ("t_moments_ms", C.c_double),
        ("spmm_launches", C.c_int64),
        ("spmm_bytes", C.c_double),
        ("kernel_launches", C.c_int64),
        ("asym_max", C.c_double),
        ("idem_err", C.c_double),
        ("sp2_iters", C.c_int32),
        ("step_kernel", C.c_int32),
        ("sp2_nnzb", C.c_int64),
        ("sp2_flops", C.c_double),
        ("sp2_bytes", C.c_double),
        ("fp32_diag_err", C.c_double),
        ("fp32_check_ms", C.c_double),
        ("sp2_flops_done", C.c_double),
        ("fp64_evals", C.c_int32),
        ("reserved_i", C.c_int32),
        ("reserved", C.c_double * 2),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("reserved")}


class TbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"status {status}: {msg}")
        self.status = status


_lib = None
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_vp = C.c_void_p


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libtb_gb300.so (building it in-tree first if allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run largetb_gb300.build.build()")
        _build.build()
    L = C.CDLL(path)
    L.tb_params_init.argtypes = [C.POINTER(TbParams)]
    L.tb_ctx_create.argtypes = [C.POINTER(TbParams), C.POINTER(_vp)]
    L.tb_ctx_destroy.argtypes = [_vp]
    L.tb_set_params.argtypes = [_vp, C.POINTER(TbParams)]
    L.tb_get_params.argtypes = [_vp, C.POINTER(TbParams)]
    L.tb_set_hamiltonian.argtypes = [_vp, C.c_int32, _i32p, _i32p, _f64p, _i32p, C.c_int32]
    L.tb_set_scc.argtypes = [_vp, C.c_int32, _i32p, _i32p, _f64p, _f64p]
    L.tb_set_geometry.argtypes = [_vp, C.c_int32, _f64p, _i32p, _f64p, C.c_double, C.c_double]
    L.tb_gershgorin.argtypes = [_vp, _vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.tb_density.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(TbReport)]
    L.tb_coulomb_shift.argtypes = [_vp, _f64p, _f64p]
    L.tb_scc_solve.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(TbReport)]
    L.tb_sp2.argtypes = [_vp, _vp, _vp, _vp, C.POINTER(TbReport)]
    L.tb_kpm_dos.argtypes = [_vp, C.c_int32, C.c_int32, C.c_uint64, C.c_int32, _vp, _vp, _vp,
                             C.POINTER(TbReport)]
    L.tb_density_stochastic.argtypes = [_vp, _vp, C.c_int32, C.c_uint64, C.c_int32, C.c_int32, _vp, _vp,
                                        C.POINTER(C.c_double), C.POINTER(TbReport)]
    L.tb_last_error.argtypes = [_vp]
    L.tb_last_error.restype = C.c_char_p
    L.tb_status_string.argtypes = [C.c_int]
    L.tb_status_string.restype = C.c_char_p
    L.tb_model_quartz.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.POINTER(_vp)]
    L.tb_model_cristobalite.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                        C.c_uint64, C.c_double, C.c_double, C.POINTER(_vp)]
    L.tb_model_sizes.argtypes = [_vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.tb_model_export.argtypes = [_vp] + [_vp] * 10
    L.tb_model_destroy.argtypes = [_vp]
    L.tb_batch_create.argtypes = [C.POINTER(TbParams), C.c_int32, C.POINTER(_vp)]
    L.tb_batch_destroy.argtypes = [_vp]
    L.tb_batch_set.argtypes = [_vp, C.c_int32, C.c_int32, _i32p, _i32p, _f64p, C.c_int32, _i32p,
                               _i32p, _f64p, _f64p]
    L.tb_batch_scc_solve.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(TbReport)]
    L.tb_batch_last_error.argtypes = [_vp]
    L.tb_batch_last_error.restype = C.c_char_p
    _f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    L.tb_mlp_features.argtypes = [C.c_int32, _f64p, _i32p, _f64p, _f32p]
    L.tb_mlp_create.argtypes = [C.c_int32, C.c_uint64, C.POINTER(_vp)]
    L.tb_mlp_destroy.argtypes = [_vp]
    L.tb_mlp_get.argtypes = [_vp, _vp, _vp]
    L.tb_mlp_set.argtypes = [_vp, _vp, _vp]
    L.tb_mlp_train.argtypes = [_vp, C.c_int32, _f32p, _f32p, C.c_int32, C.c_int32, C.c_float,
                               C.c_uint64, _vp]
    L.tb_mlp_predict.argtypes = [_vp, C.c_int32, _f32p, _f32p]
    L.tb_mlp_predict_fp32.argtypes = [_vp, C.c_int32, _f32p, _f32p]
    L.tb_mlp_grad.argtypes = [_vp, C.c_int32, _f32p, _f32p, _f32p, _vp]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def params(**kw) -> TbParams:
    """Default parameters (tb_params_init) with keyword overrides."""
    p = TbParams()
    load().tb_params_init(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


# ---------------------------------------------------------------------------
# Model builder (upstream of the boundary)
# ---------------------------------------------------------------------------
@dataclass
class Model:
    natoms: int
    rowptr: np.ndarray
    colidx: np.ndarray
    vals: np.ndarray
    orb2atom: np.ndarray
    g_rowptr: np.ndarray
    g_colidx: np.ndarray
    g_vals: np.ndarray
    q0: np.ndarray
    xyz: np.ndarray
    species: np.ndarray

    @property
    def n(self):
        return 4 * self.natoms

    @property
    def n_electrons(self):
        return float(self.q0.sum())


def _export(h) -> Model:
    L = load()
    na, n, nnz, gnnz = C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64()
    L.tb_model_sizes(h, C.byref(na), C.byref(n), C.byref(nnz), C.byref(gnnz))
    na, n, nnz, gnnz = na.value, n.value, nnz.value, gnnz.value
    m = Model(na, np.zeros(n + 1, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz),
              np.zeros(n, np.int32), np.zeros(na + 1, np.int32), np.zeros(gnnz, np.int32),
              np.zeros(gnnz), np.zeros(na), np.zeros((na, 3)), np.zeros(na, np.int32))
    L.tb_model_export(h, *[_ptr(x) for x in (m.rowptr, m.colidx, m.vals, m.orb2atom, m.g_rowptr,
                                             m.g_colidx, m.g_vals, m.q0, m.xyz, m.species)])
    L.tb_model_destroy(h)
    return m


def model_quartz(L_, M_, N_) -> Model:
    """alpha-quartz exactly as the reference builds it (withSP2_deltaH.cpp:372-1066)."""
    h = _vp()
    rc = load().tb_model_quartz(L_, M_, N_, C.byref(h))
    if rc:
        raise TbError(rc, "tb_model_quartz failed")
    return _export(h)


def model_cristobalite(nx, ny, nz, a_ang=7.16, sigma_ang=0.0, seed=0, rcut_bohr=4.0,
                       gamma_diag=1.0) -> Model:
    h = _vp()
    rc = load().tb_model_cristobalite(nx, ny, nz, a_ang, sigma_ang, seed, rcut_bohr, gamma_diag,
                                      C.byref(h))
    if rc:
        raise TbError(rc, "tb_model_cristobalite failed")
    return _export(h)


# ---------------------------------------------------------------------------
# Context
# ---------------------------------------------------------------------------
class Context:
    """One device context (tb_ctx).  Methods mirror the reference routines."""

    def __init__(self, p: TbParams | None = None, **kw):
        self._L = load()
        self.p = p if p is not None else params(**kw)
        h = _vp()
        rc = self._L.tb_ctx_create(C.byref(self.p), C.byref(h))
        if rc:
            raise TbError(rc, self._L.tb_status_string(rc).decode())
        self._h = h
        self.n = 0
        self.natoms = 0

    # -- lifecycle ------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.tb_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, allow=()):
        if rc != TB_OK and rc not in allow:
            raise TbError(rc, self._L.tb_last_error(self._h).decode())
        return rc

    def set_params(self, p: TbParams | None = None, **kw):
        if p is None:
            p = TbParams()
            self._check(self._L.tb_get_params(self._h, C.byref(p)))
            for k, v in kw.items():
                setattr(p, k, v)
        self._check(self._L.tb_set_params(self._h, C.byref(p)))
        self.p = p

    def get_params(self) -> TbParams:
        p = TbParams()
        self._check(self._L.tb_get_params(self._h, C.byref(p)))
        return p

    # -- inputs ---------------------------------------------------------
    def set_hamiltonian(self, rowptr, colidx, vals, orb2atom, natoms):
        """Assembled Htotal (seqaij i/j/a) + orbital2Atom -> device BSR."""
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        colidx = np.ascontiguousarray(colidx, np.int32)
        vals = np.ascontiguousarray(vals, np.float64)
        orb2atom = np.ascontiguousarray(orb2atom, np.int32)
        n = rowptr.shape[0] - 1
        self._check(self._L.tb_set_hamiltonian(self._h, n, rowptr, colidx, vals, orb2atom, natoms))
        self.n, self.natoms = n, natoms

    def set_scc(self, g_rowptr, g_colidx, g_vals, q0):
        """Gamma_ab CSR + neutral charges (initializeForSCF)."""
        self._check(self._L.tb_set_scc(
            self._h, self.natoms, np.ascontiguousarray(g_rowptr, np.int32),
            np.ascontiguousarray(g_colidx, np.int32), np.ascontiguousarray(g_vals, np.float64),
            np.ascontiguousarray(q0, np.float64)))

    def set_geometry(self, xyz, species, box, rcut_bohr=4.0, gamma_diag=1.0):
        """H, Gamma and q0 built on the GPU from positions (bohr) and species."""
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        species = np.ascontiguousarray(species, np.int32)
        self._check(self._L.tb_set_geometry(self._h, species.shape[0], xyz, species,
                                            np.ascontiguousarray(box, np.float64), rcut_bohr,
                                            gamma_diag))
        self.natoms = int(species.shape[0])
        self.n = 4 * self.natoms

    def set_model(self, m: Model, scc: bool = True):
        self.set_hamiltonian(m.rowptr, m.colidx, m.vals, m.orb2atom, m.natoms)
        if scc:
            self.set_scc(m.g_rowptr, m.g_colidx, m.g_vals, m.q0)

    # -- operations -----------------------------------------------------
    def gershgorin(self, shift=None):
        """GershGorinParallel (withSP2_deltaH.cpp:144-209)."""
        lo, hi = C.c_double(), C.c_double()
        sh = None if shift is None else np.ascontiguousarray(shift, np.float64)
        self._check(self._L.tb_gershgorin(self._h, _ptr(sh), C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def density(self, shift=None):
        """runKPM + computeDensityMatrix with the exact trace."""
        diagP = np.zeros(self.n)
        q = np.zeros(self.natoms)
        mom = np.zeros(self.get_params().M + 1)
        eb, mu = C.c_double(), C.c_double()
        rep = TbReport()
        sh = None if shift is None else np.ascontiguousarray(shift, np.float64)
        self._check(self._L.tb_density(self._h, _ptr(sh), _ptr(diagP), _ptr(q), C.byref(eb),
                                       C.byref(mu), _ptr(mom), C.byref(rep)))
        return dict(diagP=diagP, q=q, e_band=eb.value, mu=mu.value, moments=mom,
                    report=rep.as_dict())

    def coulomb_shift(self, q):
        """Gamma (q - q0): the gammaq of constructdeltaH."""
        V = np.zeros(self.natoms)
        self._check(self._L.tb_coulomb_shift(self._h, np.ascontiguousarray(q, np.float64), V))
        return V

    def scc_solve(self, q_init=None, raise_on_cap=True):
        q = np.zeros(self.natoms)
        diagP = np.zeros(self.n)
        eb, mu = C.c_double(), C.c_double()
        it = C.c_int32()
        rep = TbReport()
        qi = None if q_init is None else np.ascontiguousarray(q_init, np.float64)
        rc = self._check(self._L.tb_scc_solve(self._h, _ptr(qi), _ptr(q), _ptr(diagP),
                                              C.byref(eb), C.byref(mu), C.byref(it), C.byref(rep)),
                         allow=() if raise_on_cap else (TB_ERR_NOT_CONVERGED,))
        return dict(status=rc, q=q, diagP=diagP, e_band=eb.value, mu=mu.value, iters=it.value,
                    report=rep.as_dict())

    def sp2(self):
        diagP = np.zeros(self.n)
        q = np.zeros(self.natoms)
        eb = C.c_double()
        rep = TbReport()
        self._check(self._L.tb_sp2(self._h, _ptr(diagP), _ptr(q), C.byref(eb), C.byref(rep)),
                    allow=(TB_ERR_NOT_CONVERGED,))
        return dict(diagP=diagP, q=q, e_band=eb.value, report=rep.as_dict())

    def density_stochastic(self, n_probes=20, seed=0, dos_moments=1000, dos_points=2000, shift=None):
        """runKPM's stochastic DOS, mu from its area and the refined interval,
        then computeDiagonalElements' random-vector estimator."""
        diagP = np.zeros(self.n)
        q = np.zeros(self.natoms)
        mu = C.c_double()
        rep = TbReport()
        sh = None if shift is None else np.ascontiguousarray(shift, np.float64)
        self._check(self._L.tb_density_stochastic(self._h, _ptr(sh), n_probes, seed, dos_moments, dos_points,
                                                  _ptr(diagP), _ptr(q), C.byref(mu), C.byref(rep)))
        return dict(diagP=diagP, q=q, mu=mu.value, report=rep.as_dict())

    def kpm_dos(self, n_moments=1000, n_random=20, seed=0, npts=2000):
        mom = np.zeros(n_moments)
        e = np.zeros(npts)
        dos = np.zeros(npts)
        rep = TbReport()
        self._check(self._L.tb_kpm_dos(self._h, n_moments, n_random, seed, npts, _ptr(mom), _ptr(e),
                                       _ptr(dos), C.byref(rep)))
        return dict(moments=mom, energies=e, dos=dos, report=rep.as_dict())


class Batch:
    """Many structures solved together (tb_batch_*): per-structure scaling,
    mu, Anderson state and convergence on the device, one launch per
    Chebyshev step for all unconverged structures."""

    def __init__(self, models, p: TbParams | None = None, **kw):
        self._L = load()
        self.p = p if p is not None else params(**kw)
        h = _vp()
        rc = self._L.tb_batch_create(C.byref(self.p), len(models), C.byref(h))
        if rc:
            raise TbError(rc, self._L.tb_status_string(rc).decode())
        self._h = h
        self.natoms = [m.natoms for m in models]
        for i, m in enumerate(models):
            self._check(self._L.tb_batch_set(self._h, i, m.n, m.rowptr, m.colidx, m.vals, m.natoms,
                                             m.g_rowptr, m.g_colidx, m.g_vals, m.q0))

    def _check(self, rc, allow=()):
        if rc != TB_OK and rc not in allow:
            raise TbError(rc, self._L.tb_batch_last_error(self._h).decode())
        return rc

    def close(self):
        if getattr(self, "_h", None):
            self._L.tb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def scc_solve(self, q_init=None, raise_on_cap=True):
        S = len(self.natoms)
        q = np.zeros(sum(self.natoms))
        it = np.zeros(S, np.int32)
        eb = np.zeros(S)
        mu = np.zeros(S)
        rep = TbReport()
        qi = None if q_init is None else np.ascontiguousarray(q_init, np.float64)
        rc = self._check(self._L.tb_batch_scc_solve(self._h, _ptr(qi), _ptr(q), _ptr(it), _ptr(eb),
                                                    _ptr(mu), C.byref(rep)),
                         allow=() if raise_on_cap else (TB_ERR_NOT_CONVERGED,))
        offs = np.cumsum([0] + self.natoms)
        return dict(status=rc, q=[q[offs[i]:offs[i + 1]] for i in range(S)], iters=it, e_band=eb,
                    mu=mu, report=rep.as_dict())


MLP_NFEAT = 32
MLP_NPARAM = 6337


def mlp_features(xyz, species, box):
    """Per-atom radial features (tb_mlp_features), natoms x 32 float32."""
    xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1)
    species = np.ascontiguousarray(species, np.int32)
    out = np.zeros((species.shape[0], MLP_NFEAT), np.float32)
    rc = load().tb_mlp_features(species.shape[0], xyz, species, np.ascontiguousarray(box, np.float64),
                                out)
    if rc:
        raise TbError(rc, "tb_mlp_features failed")
    return out


class MLP:
    """Per-atom charge model trained and evaluated on the GPU (tb_mlp_*)."""

    def __init__(self, device=0, seed=1):
        self._L = load()
        h = _vp()
        rc = self._L.tb_mlp_create(device, seed, C.byref(h))
        if rc:
            raise TbError(rc, "tb_mlp_create failed")
        self._h = h

    def _chk(self, rc, what):
        if rc:
            raise TbError(rc, what)

    def close(self):
        if getattr(self, "_h", None):
            self._L.tb_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get(self):
        p = np.zeros(MLP_NPARAM, np.float32)
        nrm = np.zeros(2 * MLP_NFEAT, np.float32)
        self._chk(self._L.tb_mlp_get(self._h, _ptr(p), _ptr(nrm)), "tb_mlp_get")
        return p, nrm

    def set(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, np.float32)
        self._chk(self._L.tb_mlp_set(self._h, _ptr(p), _ptr(n)), "tb_mlp_set")

    def train(self, feat, target, epochs=10, batch=1024, lr=1e-3, seed=0):
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        loss = np.zeros(epochs, np.float32)
        self._chk(self._L.tb_mlp_train(self._h, target.shape[0], feat, target, epochs, batch, lr, seed,
                                       _ptr(loss)), "tb_mlp_train")
        return loss

    def predict(self, feat):
        feat = np.ascontiguousarray(feat, np.float32)
        out = np.zeros(feat.shape[0], np.float32)
        self._chk(self._L.tb_mlp_predict(self._h, feat.shape[0], feat, out), "tb_mlp_predict")
        return out

    def predict_fp32(self, feat):
        """The CUDA-core forward with FP32 layer inputs (tb_mlp_predict_fp32)."""
        feat = np.ascontiguousarray(feat, np.float32)
        out = np.zeros(feat.shape[0], np.float32)
        self._chk(self._L.tb_mlp_predict_fp32(self._h, feat.shape[0], feat, out), "tb_mlp_predict_fp32")
        return out

    def grad(self, feat, target):
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        g = np.zeros(MLP_NPARAM, np.float32)
        loss = np.zeros(1, np.float32)
        self._chk(self._L.tb_mlp_grad(self._h, target.shape[0], feat, target, g, _ptr(loss)),
                  "tb_mlp_grad")
        return g, float(loss[0])
