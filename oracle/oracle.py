"""ctypes wrapper of the FP64 CPU oracle (oracle/tb_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Only tests/,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of ``bench.py`` may
import this module; the product (``largetb_gb300``) never does.

Each wrapper names the reference function it restates (withSP2_deltaH.cpp /
withSP2.cpp of pghale/largeTB); the C file carries the line citations.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    src = os.path.join(_HERE, "tb_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(_HERE, "tb_oracle.h"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class OrcKpeParams(C.Structure):
    _fields_ = [
        ("M", C.c_int32),
        ("kernel", C.c_int32),
        ("kT", C.c_double),
        ("n_elec", C.c_double),
        ("pad", C.c_double),
        ("tol_n", C.c_double),
        ("nthreads", C.c_int32),
    ]


class OrcKpeResult(C.Structure):
    _fields_ = [
        ("lmin", C.c_double),
        ("lmax", C.c_double),
        ("a", C.c_double),
        ("b", C.c_double),
        ("mu_x", C.c_double),
        ("mu", C.c_double),
        ("e_band", C.c_double),
        ("n_elec_found", C.c_double),
        ("bisect_iters", C.c_int32),
    ]


class OrcSccParams(C.Structure):
    _fields_ = [
        ("tol", C.c_double),
        ("max_iter", C.c_int32),
        ("beta", C.c_double),
        ("history", C.c_int32),
    ]


class OrcSp2Params(C.Structure):
    _fields_ = [
        ("n_elec", C.c_double),
        ("drop_tol", C.c_double),
        ("max_iter", C.c_int32),
        ("idem_tol", C.c_double),
        ("trace_tol", C.c_double),
        ("nthreads", C.c_int32),
    ]


class OrcSp2Result(C.Structure):
    _fields_ = [
        ("iters", C.c_int32),
        ("idem_err", C.c_double),
        ("trace", C.c_double),
        ("e_band", C.c_double),
        ("nnzb", C.c_int64),
        ("lmin", C.c_double),
        ("lmax", C.c_double),
    ]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_quartz_positions.argtypes = [C.c_int, C.c_int, C.c_int, f64p, i32p]
        L.orc_quartz_cell.argtypes = [C.c_int, C.c_int, C.c_int, f64p]
        L.orc_quartz_cell.restype = None
        L.orc_cristobalite_positions.argtypes = [
            C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64, f64p, i32p]
        L.orc_cristobalite_cell.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, f64p]
        L.orc_cristobalite_cell.restype = None
        L.orc_neighbours.argtypes = [
            C.c_int, f64p, f64p, i32p, C.c_double, C.c_double, C.c_int, i32p, i32p, f64p]
        L.orc_hblock.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, f64p]
        L.orc_build_h.argtypes = [C.c_int, i32p, i32p, i32p, f64p, C.c_int, i32p, i32p, f64p]
        L.orc_build_gamma.argtypes = [
            C.c_int, i32p, i32p, f64p, C.c_int, C.c_double, i32p, i32p, f64p]
        L.orc_gershgorin.argtypes = [
            C.c_int, i32p, i32p, f64p, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_gershgorin.restype = None
        L.orc_jackson.argtypes = [C.c_int, f64p]
        L.orc_jackson.restype = None
        L.orc_kernel_autocorr.argtypes = [C.c_int, f64p]
        L.orc_kernel_autocorr.restype = None
        L.orc_step_coeffs.argtypes = [C.c_int, C.c_double, f64p]
        L.orc_step_coeffs.restype = None
        L.orc_fermi_coeffs.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, f64p]
        L.orc_fermi_coeffs.restype = None
        L.orc_quadrature_nodes.argtypes = [C.c_int, C.c_double]
        L.orc_exact_moments.argtypes = [
            C.c_int, i32p, i32p, f64p, C.c_void_p, C.c_double, C.c_double, C.c_int, f64p, C.c_int]
        L.orc_exact_moments_cols.argtypes = [
            C.c_int, i32p, i32p, f64p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int,
            C.c_int, f64p, C.c_int]
        L.orc_electron_count.argtypes = [C.c_int, f64p, f64p, C.c_double, C.c_double, C.c_int]
        L.orc_electron_count.restype = C.c_double
        L.orc_density.argtypes = [
            C.c_int, i32p, i32p, f64p, C.c_void_p, i32p, C.c_int, C.POINTER(OrcKpeParams),
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(OrcKpeResult)]
        L.orc_gamma_mult.argtypes = [C.c_int, i32p, i32p, f64p, f64p, f64p]
        L.orc_gamma_mult.restype = None
        L.orc_scc.argtypes = [
            C.c_int, i32p, i32p, f64p, i32p, C.c_int, i32p, i32p, f64p, f64p, C.c_void_p,
            C.POINTER(OrcKpeParams), C.POINTER(OrcSccParams), f64p, f64p, f64p,
            C.POINTER(C.c_int), C.POINTER(OrcKpeResult)]
        L.orc_sp2.argtypes = [
            C.c_int, i32p, i32p, f64p, i32p, C.c_int, C.POINTER(OrcSp2Params), f64p, f64p,
            i32p, f64p, f64p, C.POINTER(OrcSp2Result)]
        L.orc_anderson.argtypes = [
            C.c_int, f64p, f64p, C.c_double, C.c_int, f64p, f64p, C.POINTER(C.c_int),
            C.POINTER(C.c_int), f64p]
        L.orc_kpm_dos.argtypes = [
            C.c_int, i32p, i32p, f64p, C.c_double, C.c_double, C.c_int, C.c_int, C.c_uint64,
            C.c_int, f64p, f64p, f64p]
        L.orc_density_stochastic.argtypes = [
            C.c_int, i32p, i32p, f64p, i32p, C.c_int, C.POINTER(OrcKpeParams), C.c_int, C.c_uint64,
            C.c_int, C.c_int, f64p, f64p, C.POINTER(OrcKpeResult)]
        L.orc_dos_mu.argtypes = [C.c_int, f64p, f64p, C.c_double, C.c_int, C.POINTER(C.c_double),
                                 C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_dos_mu.restype = None
        L.orc_gauss.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_gauss.restype = C.c_double
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleError(RuntimeError):
    pass


def _check(rc, what):
    if rc != 0:
        raise OracleError(f"{what} failed with status {rc}")


# --------------------------------------------------------------------------
# Model construction (upstream of the hot path)
# --------------------------------------------------------------------------
@dataclass
class Model:
    xyz: np.ndarray       # (natoms, 3) bohr
    species: np.ndarray   # (natoms,) atomic numbers 14 / 8
    cell: np.ndarray      # (3, 3) supercell rows, bohr
    nnb: np.ndarray
    nbidx: np.ndarray
    nbvec: np.ndarray
    maxnb: int
    rowptr: np.ndarray    # CSR of H (orbitals)
    col: np.ndarray
    val: np.ndarray
    g_rowptr: np.ndarray  # CSR of Gamma (atoms)
    g_col: np.ndarray
    g_val: np.ndarray
    q0: np.ndarray        # neutral electrons per atom
    orb2atom: np.ndarray

    @property
    def natoms(self):
        return int(self.species.shape[0])

    @property
    def n(self):
        return 4 * self.natoms

    @property
    def n_elec(self):
        return float(self.q0.sum())

    def dense_h(self):
        n = self.n
        H = np.zeros((n, n))
        for i in range(n):
            H[i, self.col[self.rowptr[i]:self.rowptr[i + 1]]] = self.val[self.rowptr[i]:self.rowptr[i + 1]]
        return H


def quartz(L, M, N, maxnb=20, gamma_diag=-1.0):
    """alpha-quartz supercell exactly as the reference builds it: positions
    (initializeCoordinates), x/y-periodic halo search with 0.1 < d^2 < 16
    (getHaloAtoms), blocks (constructH) and Gamma (initializeForSCF, -Us
    diagonal)."""
    L_ = lib()
    nat = 9 * L * M * N
    xyz = np.zeros(3 * nat)
    sp = np.zeros(nat, np.int32)
    _check(L_.orc_quartz_positions(L, M, N, xyz, sp), "quartz_positions")
    cell = np.zeros(9)
    L_.orc_quartz_cell(L, M, N, cell)
    return _finish(xyz, sp, cell, np.array([1, 1, 0], np.int32), 16.0, 0.1, maxnb, gamma_diag)


def cristobalite(nx, ny, nz, a_ang=7.16, sigma_ang=0.0, seed=0, rcut_bohr=4.0, maxnb=64,
                 gamma_diag=1.0):
    """beta-cristobalite supercell, 3-D periodic, reference block model and cutoff."""
    L_ = lib()
    nat = 24 * nx * ny * nz
    xyz = np.zeros(3 * nat)
    sp = np.zeros(nat, np.int32)
    _check(L_.orc_cristobalite_positions(nx, ny, nz, a_ang, sigma_ang, seed, xyz, sp),
           "cristobalite_positions")
    cell = np.zeros(9)
    L_.orc_cristobalite_cell(nx, ny, nz, a_ang, cell)
    return _finish(xyz, sp, cell, np.array([1, 1, 1], np.int32), rcut_bohr ** 2, 0.1, maxnb,
                   gamma_diag)


def _finish(xyz, sp, cell, periodic, rcut2, rmin2, maxnb, gamma_diag):
    L_ = lib()
    nat = sp.shape[0]
    nnb = np.zeros(nat, np.int32)
    nbidx = np.zeros(nat * maxnb, np.int32)
    nbvec = np.zeros(3 * nat * maxnb)
    _check(L_.orc_neighbours(nat, xyz, cell, periodic, rcut2, rmin2, maxnb, nnb, nbidx, nbvec),
           "neighbours")
    nblk = nat + int(nnb.sum())
    rowptr = np.zeros(4 * nat + 1, np.int32)
    col = np.zeros(16 * nblk, np.int32)
    val = np.zeros(16 * nblk)
    _check(L_.orc_build_h(nat, sp, nnb, nbidx, nbvec, maxnb, rowptr, col, val), "build_h")
    g_rowptr = np.zeros(nat + 1, np.int32)
    g_col = np.zeros(nblk, np.int32)
    g_val = np.zeros(nblk)
    _check(L_.orc_build_gamma(nat, nnb, nbidx, nbvec, maxnb, gamma_diag, g_rowptr, g_col, g_val),
           "build_gamma")
    q0 = np.where(sp == 14, 4.0, 6.0)
    orb2atom = np.repeat(np.arange(nat, dtype=np.int32), 4)
    return Model(xyz.reshape(nat, 3), sp, cell.reshape(3, 3), nnb, nbidx, nbvec, maxnb, rowptr,
                 col, val, g_rowptr, g_col, g_val, q0, orb2atom)


def model_from_csr(rowptr, col, val, natoms):
    """An oracle Model around given CSR arrays (H only: no geometry/Gamma)."""
    nat = int(natoms)
    e = np.zeros(0)
    return Model(np.zeros((nat, 3)), np.zeros(nat, np.int32), np.zeros((3, 3)), np.zeros(nat, np.int32),
                 np.zeros(0, np.int32), e, 0, np.ascontiguousarray(rowptr, np.int32),
                 np.ascontiguousarray(col, np.int32), np.ascontiguousarray(val, np.float64),
                 np.zeros(nat + 1, np.int32), np.zeros(0, np.int32), e, np.zeros(nat),
                 np.repeat(np.arange(nat, dtype=np.int32), 4))


def hblock(zi, zj, x, y, z):
    out = np.zeros(16)
    _check(lib().orc_hblock(zi, zj, x, y, z, out), "hblock")
    return out.reshape(4, 4)


# --------------------------------------------------------------------------
# Hot-path restatements
# --------------------------------------------------------------------------
def gershgorin(m: Model, shift=None):
    lo, hi = C.c_double(), C.c_double()
    sh = None if shift is None else np.ascontiguousarray(shift, np.float64)
    lib().orc_gershgorin(m.n, m.rowptr, m.col, m.val, _ptr(sh), C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def jackson(M):
    g = np.zeros(M)
    lib().orc_jackson(M, g)
    return g


def kernel_autocorr(M):
    g = np.zeros(M)
    lib().orc_kernel_autocorr(M, g)
    return g


def step_coeffs(M, mu_x):
    c = np.zeros(M)
    lib().orc_step_coeffs(M, mu_x, c)
    return c


def fermi_coeffs(M, mu_x, beta_x, nq=None):
    if nq is None:
        nq = lib().orc_quadrature_nodes(M, beta_x)
    c = np.zeros(M)
    lib().orc_fermi_coeffs(M, mu_x, beta_x, nq, c)
    return c


def quadrature_nodes(M, beta_x):
    return int(lib().orc_quadrature_nodes(M, beta_x))


def exact_moments(m: Model, a, b, nmom, shift=None, nthreads=0):
    d = np.zeros(nmom * m.n)
    sh = None if shift is None else np.ascontiguousarray(shift, np.float64)
    _check(lib().orc_exact_moments(m.n, m.rowptr, m.col, m.val, _ptr(sh), a, b, nmom, d, nthreads),
           "exact_moments")
    return d.reshape(nmom, m.n)


def exact_moments_cols(m: Model, a, b, nmom, c_begin, c_end, shift=None, nthreads=0):
    """Moments of identity columns c_begin..c_end-1 only (a bounded timing sample)."""
    d = np.zeros(nmom * m.n)
    sh = None if shift is None else np.ascontiguousarray(shift, np.float64)
    _check(lib().orc_exact_moments_cols(m.n, m.rowptr, m.col, m.val, _ptr(sh), a, b, nmom, c_begin,
                                        c_end, d, nthreads), "exact_moments_cols")
    return d.reshape(nmom, m.n)


def kpe_params(M=200, kT=0.01, n_elec=0.0, kernel=0, pad=0.0, tol_n=1e-9, nthreads=0):
    return OrcKpeParams(M, kernel, kT, n_elec, pad, tol_n, nthreads)


def density(m: Model, p: OrcKpeParams, shift=None, want_d=False):
    """runKPM + computeDensityMatrix with exact trace (see tb_oracle.h)."""
    n = m.n
    diagP = np.zeros(n)
    q = np.zeros(m.natoms)
    mom = np.zeros(p.M + 1)
    d = np.zeros((p.M + 1) * n) if want_d else None
    res = OrcKpeResult()
    sh = None if shift is None else np.ascontiguousarray(shift, np.float64)
    rc = lib().orc_density(n, m.rowptr, m.col, m.val, _ptr(sh), m.orb2atom, m.natoms, C.byref(p),
                           _ptr(diagP), _ptr(q), _ptr(mom), _ptr(d), C.byref(res))
    _check(rc, "density")
    out = dict(diagP=diagP, q=q, moments=mom, lmin=res.lmin, lmax=res.lmax, a=res.a, b=res.b,
               mu_x=res.mu_x, mu=res.mu, e_band=res.e_band, n_elec_found=res.n_elec_found,
               bisect_iters=res.bisect_iters)
    if want_d:
        out["d"] = d.reshape(p.M + 1, n)
    return out


def gamma_mult(m: Model, dq):
    out = np.zeros(m.natoms)
    lib().orc_gamma_mult(m.natoms, m.g_rowptr, m.g_col, m.g_val,
                         np.ascontiguousarray(dq, np.float64), out)
    return out


def scc(m: Model, p: OrcKpeParams, tol=1e-6, max_iter=100, beta=0.3, history=6, q_init=None):
    """The working SCC loop the reference sketches (withSP2_deltaH.cpp:1820-1840)."""
    q = np.zeros(m.natoms)
    diagP = np.zeros(m.n)
    hist = np.zeros(max_iter)
    it = C.c_int(0)
    res = OrcKpeResult()
    s = OrcSccParams(tol, max_iter, beta, history)
    qi = None if q_init is None else np.ascontiguousarray(q_init, np.float64)
    rc = lib().orc_scc(m.n, m.rowptr, m.col, m.val, m.orb2atom, m.natoms, m.g_rowptr, m.g_col,
                       m.g_val, m.q0, _ptr(qi), C.byref(p), C.byref(s), q, diagP, hist,
                       C.byref(it), C.byref(res))
    return dict(status=rc, q=q, diagP=diagP, iters=it.value, dq_hist=hist[: it.value],
                e_band=res.e_band, mu=res.mu, mu_x=res.mu_x, a=res.a, b=res.b)


class Anderson:
    """The oracle's Anderson mixer (orc_anderson) with its ring of past
    (q_in, residual) pairs held here, so a caller can run orc_scc's loop one
    density evaluation at a time and save or restore the mixer between them."""

    def __init__(self, natoms, beta=0.2, history=16):
        self.natoms, self.beta, self.history = natoms, beta, history
        h = max(history, 1)
        self.hq = np.zeros(h * natoms)
        self.hr = np.zeros(h * natoms)
        self.count, self.head = C.c_int(0), C.c_int(0)

    def step(self, q_in, r):
        out = np.zeros(self.natoms)
        _check(lib().orc_anderson(self.natoms, np.ascontiguousarray(q_in, np.float64),
                                  np.ascontiguousarray(r, np.float64), self.beta, self.history,
                                  self.hq, self.hr, C.byref(self.count), C.byref(self.head), out),
               "anderson")
        return out

    def state(self):
        return dict(hq=self.hq.copy(), hr=self.hr.copy(), count=self.count.value,
                    head=self.head.value)

    def restore(self, st):
        self.hq[:] = st["hq"]
        self.hr[:] = st["hr"]
        self.count.value, self.head.value = int(st["count"]), int(st["head"])


class SccLoop:
    """orc_scc's loop (withSP2_deltaH.cpp:1820-1840 made to converge) one
    density evaluation at a time: the same C routines in the same order, so
    its iterates are bit-identical to orc_scc's.  step() evaluates the density
    at the current input charges, records the residual, mixes, and returns
    (iteration, q_in, density result, max |q_out - q_in|).  state()/restore()
    save and reload everything the next step depends on."""

    def __init__(self, m: Model, p: OrcKpeParams, beta=0.2, history=16, q_init=None):
        self.m, self.p = m, p
        self.mix = Anderson(m.natoms, beta, history)
        self.it = 0
        self.q_in = np.array(m.q0 if q_init is None else q_init, np.float64)

    def step(self, mix=True):
        m = self.m
        self.it += 1
        V = gamma_mult(m, self.q_in - m.q0)
        r = density(m, self.p, shift=V[m.orb2atom])
        res = r["q"] - self.q_in
        q_in = self.q_in
        if mix:
            self.q_in = self.mix.step(q_in, res)
        return self.it, q_in, r, float(np.abs(res).max())

    def state(self):
        return dict(it=self.it, q_in=self.q_in.copy(), **self.mix.state())

    def restore(self, st):
        self.it = int(st["it"])
        self.q_in = np.array(st["q_in"], np.float64)
        self.mix.restore(st)

def sp2(m: Model, drop_tol=1e-5, max_iter=40, idem_tol=1e-10, trace_tol=0.0, nthreads=0):
    """Thresholded block SP2 (getSP2/computeAlphas restated as matrix purification)."""
    p = OrcSp2Params(m.n_elec, drop_tol, max_iter, idem_tol, trace_tol, nthreads)
    diagP = np.zeros(m.n)
    q = np.zeros(m.natoms)
    br = np.zeros(max_iter + 1, np.int32)
    ih = np.zeros(max_iter + 1)
    th = np.zeros(max_iter + 1)
    r = OrcSp2Result()
    _check(lib().orc_sp2(m.n, m.rowptr, m.col, m.val, m.orb2atom, m.natoms, C.byref(p), diagP, q,
                         br, ih, th, C.byref(r)), "sp2")
    return dict(diagP=diagP, q=q, iters=r.iters, idem_err=r.idem_err, trace=r.trace,
                e_band=r.e_band, nnzb=r.nnzb, lmin=r.lmin, lmax=r.lmax,
                branches=br[: r.iters], idem_hist=ih[: r.iters + 1], trace_hist=th[: r.iters + 1])


def density_stochastic(m: Model, p: OrcKpeParams, n_random=20, seed=0, dos_moments=1000,
                       dos_points=2000):
    """runKPM (stochastic DOS, mu from its area, refined a, b) +
    computeDensityMatrix's ratio estimator (see tb_oracle.h)."""
    diagP = np.zeros(m.n)
    q = np.zeros(m.natoms)
    res = OrcKpeResult()
    _check(lib().orc_density_stochastic(m.n, m.rowptr, m.col, m.val, m.orb2atom, m.natoms, C.byref(p),
                                        n_random, seed, dos_moments, dos_points, diagP, q,
                                        C.byref(res)), "density_stochastic")
    return dict(diagP=diagP, q=q, mu=res.mu, mu_x=res.mu_x, a=res.a, b=res.b, lmin=res.lmin,
                lmax=res.lmax)


def dos_mu(energies, dos, n_elec, n):
    mu, mi, a, b = C.c_double(), C.c_int(), C.c_double(), C.c_double()
    lib().orc_dos_mu(len(dos), np.ascontiguousarray(energies, np.float64), np.ascontiguousarray(dos, np.float64),
                     n_elec, n, C.byref(mu), C.byref(mi), C.byref(a), C.byref(b))
    return dict(mu=mu.value, mu_index=mi.value, a=a.value, b=b.value)


def kpm_dos(m: Model, a, b, nmom=1000, n_random=20, seed=0, npts=2000):
    mom = np.zeros(nmom)
    e = np.zeros(npts)
    dos = np.zeros(npts)
    _check(lib().orc_kpm_dos(m.n, m.rowptr, m.col, m.val, a, b, nmom, n_random, seed, npts, mom, e,
                             dos), "kpm_dos")
    return mom, e, dos


def gauss(seed, index):
    return lib().orc_gauss(seed, index)
