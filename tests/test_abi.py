"""The C-ABI library builds, loads and exports every declared symbol (CPU)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(tb_\w+)\s*\(", txt, re.M))
    return names


def test_every_declared_symbol_is_exported():
    import largetb_gb300 as T
    L = T.load()
    names = _declared()
    assert len(names) >= 20
    for nm in sorted(names):
        assert hasattr(L, nm), nm
    out = subprocess.run(["nm", "-D", "--defined-only", T.api.library_path()], capture_output=True,
                         text=True).stdout
    for nm in names:
        assert re.search(r"\bT " + nm + r"\b", out), nm


def test_struct_layouts_match():
    import largetb_gb300 as T
    p = T.params()
    assert p.struct_size == C.sizeof(T.TbParams)
    assert p.M == 200 and p.mix_history == 16 and p.scc_tol == 1e-6


def test_no_device_fails_loudly():
    import largetb_gb300 as T
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(T.TbError) as e:
        T.Context()
    assert e.value.status == T.api.TB_ERR_NO_DEVICE


def test_bad_params_rejected_before_device():
    import largetb_gb300 as T
    L = T.load()
    p = T.params(M=1)
    h = C.c_void_p()
    assert L.tb_ctx_create(C.byref(p), C.byref(h)) == T.api.TB_ERR_INVALID_ARG
    p = T.params(column_block=100)
    assert L.tb_ctx_create(C.byref(p), C.byref(h)) == T.api.TB_ERR_INVALID_ARG
    p = T.params(fp32_kernel=5)
    assert L.tb_ctx_create(C.byref(p), C.byref(h)) == T.api.TB_ERR_INVALID_ARG
    p = T.params(mode=2)
    assert L.tb_ctx_create(C.byref(p), C.byref(h)) == T.api.TB_ERR_INVALID_ARG
    p = T.params()
    p.struct_size = 8
    assert L.tb_ctx_create(C.byref(p), C.byref(h)) == T.api.TB_ERR_INVALID_ARG


def test_peaks_helper_builds_beside_the_library():
    """libtb_peaks.so (the FP64 FMA-rate probe the benchmark uses) is built by
    the same build step, exports its one entry and refuses a null output
    without touching a device."""
    from largetb_gb300 import build as B
    B.build()  # incremental: compiles only what is missing or stale
    path = B.PEAKS_LIB
    assert os.path.exists(path)
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    assert re.search(r"\bT tb_peak_fp64_fma\b", out)
    L = C.CDLL(path)
    assert L.tb_peak_fp64_fma(0, None) != 0
