"""The allocation-free entry point tb_moments_noalloc, through the C-ABI.

It serves callers that cannot allocate device memory (their device memory
belongs to their own pool, or they run under a fixed budget): the matrix and
the output are already on the device, and the recurrence's scratch is a
static device array.  Its moments must equal those of the allocating entry
point tb_density on the same matrix (FP64 both: within 1e-9 per unit trace),
on two calls in a row -- the second call reuses the scratch the first left
behind.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(L):
    f = L.tb_moments_noalloc
    f.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                  C.c_int32, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_moments_match_allocating_entry(gpu):
    import torch
    T = gpu
    m = T.model_cristobalite(2, 2, 2, sigma_ang=0.05, seed=1001)
    M = 120
    with T.Context(M=M, precision=T.PREC_FP64, device=0) as c:
        c.set_model(m)
        ref = c.density()
    a, b = ref["report"]["a"], ref["report"]["b"]
    dev = torch.device("cuda:0")
    rp = torch.from_numpy(m.rowptr).to(dev)
    ci = torch.from_numpy(m.colidx).to(dev)
    v = torch.from_numpy(m.vals).to(dev)
    out = torch.empty(M + 1, dtype=torch.float64, device=dev)
    f = _entry(T.load())
    got = []
    for _ in range(2):
        out.fill_(12345.0)  # stale output must be cleared by the call
        torch.cuda.synchronize()
        rc = f(m.n, rp.data_ptr(), ci.data_ptr(), v.data_ptr(), a, b, M, out.data_ptr(), None)
        assert rc == 0
        got.append(out.cpu().numpy().copy())
    for g in got:
        np.testing.assert_allclose(g, ref["moments"], atol=1e-9 * m.n, rtol=0)
    np.testing.assert_allclose(got[1], got[0], atol=1e-9 * m.n, rtol=0)
    # beyond the static scratch (TB_NOALLOC_MAX_N = 8192): a clear refusal, no GPU work
    rc = f(8192 + 1, rp.data_ptr(), ci.data_ptr(), v.data_ptr(), a, b, M, out.data_ptr(), None)
    assert rc == T.api.TB_ERR_UNSUPPORTED
