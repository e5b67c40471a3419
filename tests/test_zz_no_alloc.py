"""The allocation-free entry point tb_moments_noalloc, through the C-ABI.

It serves callers that cannot allocate device memory: codes whose device
memory belongs to their own pool or allocator, or that run under a fixed
budget.  The matrix and the output are already on the device, and the
recurrence's scratch is a static device array.  Its moments must equal those
of the allocating entry point tb_density and of the FP64 oracle on the same
matrix (FP64 throughout: within 1e-9 per unit of trace), on two calls in a
row -- the second call reuses the scratch the first left behind -- and the
second call must leave the device's free memory unchanged.  Sizes: a full
2x2x2 cell (768 orbitals, a multiple of the 64-column slab), a 1x1x1 cell
(96 orbitals: one ragged slab) and the largest n the scratch holds (8192).
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 8192  # TB_NOALLOC_MAX_N


def _entry(L):
    f = L.tb_moments_noalloc
    f.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                  C.c_int32, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _chain_csr(natoms, seed):
    """A 1-D periodic chain of 4-orbital sites, each coupled to its neighbours
    at distance 1 and 2 by random 4x4 blocks (symmetric H, sorted CSR)."""
    rng = np.random.default_rng(seed)
    n = 4 * natoms
    blocks = {}
    for i in range(natoms):
        d = rng.normal(size=(4, 4))
        blocks[(i, i)] = (d + d.T) / 2 - 2.0 * np.eye(4)
        for s in (1, 2):
            j = (i + s) % natoms
            o = 0.3 * rng.normal(size=(4, 4)) / s
            blocks[(i, j)] = o
            blocks[(j, i)] = o.T
    rows = [[] for _ in range(n)]
    for (i, j), B in blocks.items():
        for r in range(4):
            for c in range(4):
                rows[4 * i + r].append((4 * j + c, B[r, c]))
    rowptr = np.zeros(n + 1, np.int32)
    col, val = [], []
    for i, row in enumerate(rows):
        row.sort()
        col += [c for c, _ in row]
        val += [v for _, v in row]
        rowptr[i + 1] = len(col)
    return rowptr, np.array(col, np.int32), np.array(val)


def _run_twice(T, rowptr, colidx, vals, a, b, M):
    import torch
    dev = torch.device("cuda:0")
    rp = torch.from_numpy(rowptr).to(dev)
    ci = torch.from_numpy(colidx).to(dev)
    v = torch.from_numpy(vals).to(dev)
    out = torch.empty(M + 1, dtype=torch.float64, device=dev)
    f = _entry(T.load())
    n = len(rowptr) - 1
    got, free = [], []
    for _ in range(2):
        out.fill_(12345.0)  # a stale output must be cleared by the call
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        rc = f(n, rp.data_ptr(), ci.data_ptr(), v.data_ptr(), a, b, M, out.data_ptr(), None)
        assert rc == 0, rc
        got.append(out.cpu().numpy().copy())
    free.append(torch.cuda.mem_get_info()[0])
    # the second call (scratch set up by the first) must not change free device memory
    assert free[2] == free[1]
    return got, (rp, ci, v, out, f)


def test_noalloc_moments_match_allocating_entry(gpu):
    from oracle import oracle as O
    T = gpu
    M = 120
    for cells in ((2, 2, 2), (1, 1, 1)):
        m = T.model_cristobalite(*cells, sigma_ang=0.05, seed=1001)
        with T.Context(M=M, precision=T.PREC_FP64, device=0) as c:
            c.set_model(m)
            ref = c.density()
        a, b = ref["report"]["a"], ref["report"]["b"]
        got, keep = _run_twice(T, m.rowptr, m.colidx, m.vals, a, b, M)
        om = O.model_from_csr(m.rowptr, m.colidx, m.vals, m.natoms)
        orc = O.exact_moments(om, a, b, M + 1).sum(axis=1)
        for g in got:
            np.testing.assert_allclose(g, ref["moments"], atol=1e-9 * m.n, rtol=0)
            np.testing.assert_allclose(g, orc, atol=1e-9 * m.n, rtol=0)
        np.testing.assert_allclose(got[1], got[0], atol=1e-9 * m.n, rtol=0)
    # beyond the static scratch: a clear refusal, no GPU work
    rp, ci, v, out, f = keep
    rc = f(MAX_N + 1, rp.data_ptr(), ci.data_ptr(), v.data_ptr(), a, b, M, out.data_ptr(), None)
    assert rc == T.api.TB_ERR_UNSUPPORTED


def test_noalloc_at_maximum_size(gpu):
    from oracle import oracle as O
    T = gpu
    M = 24
    rowptr, colidx, vals = _chain_csr(MAX_N // 4, seed=7)
    om = O.model_from_csr(rowptr, colidx, vals, MAX_N // 4)
    lo, hi = O.gershgorin(om)
    a, b = (hi - lo) / 2 * 1.01, (hi + lo) / 2
    got, _ = _run_twice(T, rowptr, colidx, vals, a, b, M)
    orc = O.exact_moments(om, a, b, M + 1).sum(axis=1)
    for g in got:
        np.testing.assert_allclose(g, orc, atol=1e-9 * MAX_N, rtol=0)
    assert got[0][0] == MAX_N
