"""In-tree build of libtb_gb300.so (the C-ABI of include/largetb.h).

Every translation unit is compiled by nvcc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into
largetb_gb300/_build/libtb_gb300.so with the static CUDA runtime.  Host C++ is
built with -ffp-contract=off so x86-64 and aarch64 hosts round alike.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtb_gb300.so")
# measurement helper beside the library (not part of include/largetb.h)
PEAKS_SRC = "tb_peaks.cu"
PEAKS_LIB = os.path.join(OUT_DIR, "libtb_peaks.so")
SOURCES = ["tb_api.cpp", "tb_model.cpp", "tb_kpe.cu", "tb_sp2.cu", "tb_dos.cu", "tb_batch.cu", "tb_geom.cu", "tb_mlp.cu", "tb_noalloc.cu", "tb_pipe.cu", "tb_mlp_tc.cu"]
HEADERS = ["tb_internal.h", "tb_abi_guard.h", "tb_f32x2.cuh", os.path.join("..", "..", "include", "largetb.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build largetb_gb300")


def _flags():
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []
    jobs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, s.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *hdrs]):
            jobs.append([nvcc(), *_flags(), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or res.returncode != 0:
                print(" ".join(cmd))
                print(res.stdout + res.stderr)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            print(" ".join(cmd))
            print(res.stdout + res.stderr)
            raise RuntimeError("link of libtb_gb300.so failed")
    psrc = os.path.join(CSRC, PEAKS_SRC)
    if os.path.exists(psrc) and (force or _stale(PEAKS_LIB, [psrc])):
        cmd = [nvcc(), *_flags(), "-shared", "-cudart", "static", "-o", PEAKS_LIB, psrc]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            print(" ".join(cmd))
            print(res.stdout + res.stderr)
            raise RuntimeError("build of libtb_peaks.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
