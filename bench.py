"""Benchmark: seconds per converged SCC solve of 6x6x6 beta-cristobalite.

Workload (one "step"): a full self-consistent-charge solve of a 6x6x6
beta-cristobalite supercell (5184 atoms, 20736 sp3 orbitals, sigma = 0.05 A
Gaussian displacements, seed 2002, reference block model, 4-bohr cutoff),
KPE order M = 400, Jackson damping, kT = 0.01 Ha, exact trace over all 20736
identity columns, Anderson mixing until max|q_out - q_in| < 1e-6 e.  The
fast form (FP32 recurrence, FP64 moments) is the timed arm; the plain FP64
GPU form is solved once beside it.

  value  device time per solve (CUDA events on the library's stream), the
         Hamiltonian already resident in HBM
  e2e    the same solve through the public C-ABI with host buffers: CSR
         upload, BSR conversion, solve, charges back to the host
  roofline  the Chebyshev SpMM step kernel: algorithmic bytes
         nnzb (16 s + 4) + (nb + 1) 4 + 3 n B s per slab step over the
         event-timed moment passes, against MEASURED_PEAKS.json hbm_gbs
  cpu_baseline  the FP64 CPU oracle (all host threads) on a bounded sample

After the timed region the line also carries the plain FP64 solve (with its
flop rate against the FP64 FMA rate measured by libtb_peaks.so), the
distances to the FP64 oracle's fixture, the SP2 purification of 4x4x4, the
64-cell batch, the 8x8x8 learned-start solve and the reference's logged
stages on the workload of its log (8x8x8 alpha-quartz, 500 vectors).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(workload="beta-cristobalite 6x6x6 SCC solve", cells=[6, 6, 6], atoms=5184,
                orbitals=20736, sigma_ang=0.05, seed=2002, M=400, kT=0.01, scc_tol=1e-6,
                cutoff_bohr=4.0, mixer="anderson(16, 0.2); 0.1 from the learned start",
                trace="exact, all identity columns",
                l2="GPU arm: a 256 MB buffer is written between timed steps (L2 flush)",
                parallelism="replicas (one independent solve per GPU)")
METRIC = "s per converged SCC solve (5184 atoms, |dq|<1e-6 e)"


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


STEP_KERNELS = {1: "k_cheb_f32_staged", 2: "k_cheb_f32_persistent", 3: "k_cheb_f32_pipe", 4: "k_cheb_f32_pipe"}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per step launch from one
# ncu capture of that kernel on the 6x6x6 workload: (step kernel, slab width) -> bytes
DRAM_TRAFFIC_6X6X6 = {(4, 20736): 5188.6e6, (4, 3456): 829.5e6, (4, 1024): 215.8e6, (1, 512): 91.2e6}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


_FP64_PEAK = {}


def fp64_peak(device):
    """FP64 FMA rate of the CUDA cores (TFLOP/s), measured by libtb_peaks.so
    (eight register-resident FMA chains per thread, best of three launches):
    the roofline of the FP64 paths.  None if the helper is missing."""
    if device not in _FP64_PEAK:
        import ctypes
        path = os.path.join(ROOT, "largetb_gb300", "_build", "libtb_peaks.so")
        val = None
        if os.path.exists(path):
            out = ctypes.c_double(0.0)
            if ctypes.CDLL(path).tb_peak_fp64_fma(int(device), ctypes.byref(out)) == 0:
                val = out.value
        _FP64_PEAK[device] = val
    return _FP64_PEAK[device]


def fp64_roofline(flop, seconds, device):
    rate = flop / seconds / 1e12
    pk = fp64_peak(device)
    return {"fp64_tflops": rate, "fp64_fma_peak_tflops": pk, "frac_fp64_peak": rate / pk if pk else None,
            "flop": flop}


class Clocks:
    """nvidia-smi sampling during the timed region (read-only queries)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # raw samples: LARGETB_CLOCKS_DIR if set, else the system temporary directory
        out = os.environ.get("LARGETB_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, f"clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def l2_flush(device):
    """Write a buffer larger than the 129 MB L2 between timed steps."""
    import torch
    buf = getattr(l2_flush, "buf", None)
    if buf is None:
        buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{device}")
        l2_flush.buf = buf
    buf.zero_()
    torch.cuda.synchronize(device)


def oracle_fixture(cells):
    """The FP64-oracle SCC of this cell, run to convergence on the CPU and
    committed as a fixture (tests/golden/make_scc_oracle.py), or None."""
    path = os.path.join(ROOT, "tests", "golden", "scc_oracle_%dx%dx%d.npz" % tuple(cells))
    return np.load(path) if os.path.exists(path) else None


def scc_iterations(cells):
    """SCC iterations of the FP64 oracle to |dq| < 1e-6 e on this cell (the
    committed fixture), or None when the cell has no fixture."""
    fx = oracle_fixture(cells)
    return None if fx is None else int(fx["iters"])


def cpu_sample(model_o, M, n_threads, iters, iters_src, cols=None):
    """FP64 oracle on a bounded sample of the workload, timed: the complete
    Chebyshev recurrence (all M + 1 moments) of a contiguous block of
    identity columns.  Every column costs the same (same matrix, same
    steps), so columns scale it exactly to one density evaluation; the
    oracle's own SCC iteration count on this cell scales that to a solve."""
    from oracle import oracle as O
    lo, hi = O.gershgorin(model_o)
    a, b = (hi - lo) / 2, (hi + lo) / 2
    cols = min(model_o.n, cols or 256 * n_threads)
    t0 = time.perf_counter()
    O.exact_moments_cols(model_o, a, b, M + 1, 0, cols, nthreads=n_threads)
    dt = time.perf_counter() - t0
    per_eval = dt * (model_o.n / cols)
    return dict(value=per_eval * iters, unit="s", cores=n_threads, kind="port",
                sample=(f"FP64 oracle, complete {M}-step recurrences of {cols} of {model_o.n} identity "
                        f"columns in {dt:.2f} s on {n_threads} threads, x {model_o.n / cols:.2f} columns = "
                        f"{per_eval:.1f} s per density evaluation, x {iters} SCC iterations ({iters_src})"))


def measured_oracle_solve(cells):
    """The one full FP64-oracle SCC solve of this cell that was run end to
    end (to build the fixture): its wall time, iterations and threads."""
    fx = oracle_fixture(cells)
    if fx is None:
        return None
    it = int(fx["iters"])
    return {"s": float(np.sum(fx["eval_s"][:it])), "iters": it, "threads": int(fx["threads"]),
            "host": "the x86-64 development container that generated the fixture"}


def run_reference(args, ws, rank):
    """The reference arm: the reference's own CPU code cannot be built here
    (PETSc and MPI are external libraries absent from this image), so its
    FP64 restatement (oracle/) runs on all host threads.  Each step times a
    bounded sample of the workload (complete recurrences of a block of
    identity columns) scaled to a solve with the oracle's own iteration
    count on this cell."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    c = WORKLOAD["cells"]
    mo = O.cristobalite(*c, sigma_ang=WORKLOAD["sigma_ang"], seed=WORKLOAD["seed"])
    nth = os.cpu_count() or 1
    iters = scc_iterations(c)
    src = "the FP64 oracle's converged SCC of this cell, committed fixture"
    if iters is None:  # no fixture for this cell: the oracle's own SCC on the 2x2x2 cell
        small = O.cristobalite(2, 2, 2, sigma_ang=WORKLOAD["sigma_ang"], seed=WORKLOAD["seed"])
        iters = O.scc(small, O.kpe_params(M=WORKLOAD["M"], kT=WORKLOAD["kT"], n_elec=small.n_elec,
                                         nthreads=nth), tol=1e-6, max_iter=100, beta=0.2, history=16)["iters"]
        src = "the FP64 oracle's SCC on the 2x2x2 cell"
    vals = []
    for i in range(args.warmup + args.steps):
        # warm-up steps take a quarter of the sample; each timed step ~3 s on 16 cores
        cb = cpu_sample(mo, WORKLOAD["M"], nth, iters, src, cols=(16 if i < args.warmup else 64) * nth)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = statistics.mean(vals)
    cb["value"] = v
    cb["kind"] = "port"
    cb["sample"] += f"; mean of {args.steps} timed samples"
    full = measured_oracle_solve(c)
    line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(WORKLOAD), "impl": "reference", "cpu_baseline": cb,
            "oracle_full_solve_measured": full,
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batch_models(T, count=64, seed=4004):
    """64 beta-cristobalite supercells, each side uniform in {2,3,4}, sigma
    uniform in [0.02, 0.12] A, structure i seeded with seed + i."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        dims = [int(x) for x in rng.integers(2, 5, size=3)]
        sig = float(rng.uniform(0.02, 0.12))
        out.append((dims, sig, T.model_cristobalite(*dims, sigma_ang=sig, seed=seed + i)))
    return out


def run_batch_bench(args, T, dev, rank):
    M = 300
    ms = batch_models(T)[: args.structures]
    models = [m for _, _, m in ms]
    atoms = np.array([m.natoms for m in models])
    b = T.Batch(models, M=M, device=dev)
    for _ in range(args.warmup):
        b.scc_solve()
    ts, am, gbs = [], [], []
    for _ in range(args.steps):
        l2_flush(dev)
        r = b.scc_solve()
        t = r["report"]["t_total_ms"] / 1e3
        ts.append(t)
        am.append(float((atoms * M * r["iters"]).sum()) / t)
        # algorithmic bytes of the Chebyshev steps over the event-timed moment phase
        gbs.append(r["report"]["spmm_bytes"] / (r["report"]["t_moments_ms"] / 1e3) / 1e9)
    b.close()
    peak, src = peaks()
    # the single-structure forms looped over structures
    def loop(prec, idx):
        tot_t, tot_am = 0.0, 0.0
        for i in idx:
            c = T.Context(M=M, precision=prec, device=dev)
            c.set_model(models[i])
            c.scc_solve()  # warm-up (slab-width autotune)
            s = c.scc_solve()
            t = s["report"]["t_total_ms"] / 1e3
            tot_t += t
            tot_am += atoms[i] * M * s["iters"]
            c.close()
        return tot_am / tot_t, tot_t
    loop32 = t32 = loop64 = t64 = None
    sub = [int(i) for i in np.argsort(atoms)[:: max(1, len(models) // 4)][:4]]
    if not args.no_plain:  # the single-structure loops beside the batch
        loop32, t32 = loop(T.PREC_FP32, range(len(models)))
        loop64, t64 = loop(T.PREC_FP64, sub)
    out = {
            "metric": f"atoms*moments/s, batched SCC of {len(models)} uneven cristobalite cells (M = 300)",
            "value": statistics.mean(am), "unit": "atom-moments/s", "higher_is_better": True,
            "s_per_batch_solve": statistics.mean(ts), "structures": len(models),
            "atoms_total": int(atoms.sum()), "atoms_min": int(atoms.min()), "atoms_max": int(atoms.max()),
            "scc_iterations": [int(x) for x in r["iters"]],
            "step_kernel": {"name": "k_cheb_f32_pipe<batch>", "GBps_algorithmic": statistics.mean(gbs),
                            "frac": statistics.mean(gbs) / peak, "peak_GBps": peak, "peak_source": src,
                            "timed": "moment phase (steps and per-step finalize), CUDA events"},
            "loop_fp32_single": {"value": loop32, "s_total": t32},
            "loop_plain_fp64_single": {"value": loop64, "structures": sub, "s_total_subset": t64},
            "speedup_vs_loop_plain_fp64": statistics.mean(am) / loop64 if loop64 else None,
            "speedup_vs_loop_fp32": statistics.mean(am) / loop32 if loop32 else None,
            "config": {"dims": [d for d, _, _ in ms], "sigma_ang": [round(sg, 4) for _, sg, _ in ms],
                       "seed": 4004, "M": M, "kT": 0.01, "scc_tol": 1e-6}}
    if rank == 0 and args.batch:
        print(json.dumps(out), flush=True)
    return out


# The reference's own stage times on its own workload (testrun_scf2:2,6,8):
# alpha-quartz 8x8x8 (4608 atoms, 18432 orbitals), 500 random vectors, on
# about 64 Cray XE cores (18432 orbitals / 288 local rows, testrun_scf2:4).
REFERENCE_LOGGED = {"log": "testrun_scf2", "kpm_dos_s": 43.2715, "first_density_s": 13.7305,
                    "ranks_inferred": 64, "machine": "Blue Waters Cray XE (FP64 PETSc)"}


def run_reference_stages(args, T, dev, rank):
    """The reference's two logged stages, on the workload of its log: runKPM
    (500 Gaussian vectors x 1000 Jackson moments of 8x8x8 alpha-quartz,
    withSP2_deltaH.cpp:1579-1648) against tb_kpm_dos with the same sizes,
    and computeDensityMatrix (1401-1412: computeAlphas' SP2 traces and
    computeDiagonalElements, 500 vectors each through getKPE at M = 200 with
    step coefficients, 1068-1399) against the density part of
    tb_density_stochastic (mu from the DOS area, the interval refined from
    its support, 500 probes at M = 200, kT = 0), FP64, on one GPU, times
    from CUDA events."""
    m = T.model_quartz(8, 8, 8)
    c = T.Context(M=200, kT=0.0, precision=T.PREC_FP64, device=dev)
    c.set_model(m)
    c.kpm_dos(n_moments=1000, n_random=500, seed=1, npts=2000)  # warm-up
    l2_flush(dev)
    t_kpm = c.kpm_dos(n_moments=1000, n_random=500, seed=2, npts=2000)["report"]["t_total_ms"] / 1e3
    l2_flush(dev)
    r = c.density_stochastic(n_probes=500, seed=3, dos_moments=1000, dos_points=2000)
    c.close()
    t_all = r["report"]["t_total_ms"] / 1e3
    ref = REFERENCE_LOGGED
    nnzb = int(m.rowptr[-1]) // 16
    cols = (500 + 63) // 64 * 64  # the probes in whole 64-column slabs
    return {"metric": "s per stage, the reference's logged workload (8x8x8 alpha-quartz, 500 vectors)",
            "config": {"cells": [8, 8, 8], "atoms": m.natoms, "orbitals": m.n, "vectors": 500,
                       "dos_moments": 1000, "M": 200, "kT": 0.0, "precision": "fp64"},
            "kpm_dos_s": t_kpm, "density_s": t_all - t_kpm, "dos_plus_density_s": t_all,
            "electrons": float(r["q"].sum()), "n_electrons": m.n_electrons,
            "reference_logged": ref,
            "kpm_dos_roofline": fp64_roofline(999.0 * nnzb * 32.0 * cols, t_kpm, dev),
            "ratio_kpm_dos": ref["kpm_dos_s"] / t_kpm,
            "ratio_density": ref["first_density_s"] / max(t_all - t_kpm, 1e-9)}


def run_learned_eval(args, T, dev, rank):
    """Learned SCC start on an 8x8x8 cell (12288 atoms, 49152 orbitals),
    sigma 0.08 A, M = 200 (the training M), FP32 form: iterations and time to
    |dq| < 1e-6 e from the neutral charges and from the MLP prediction."""
    from largetb_gb300 import learned
    cells = args.cells or [8, 8, 8]
    m = T.model_cristobalite(*cells, sigma_ang=0.08, seed=8008)
    mlp = learned.load(device=dev)
    box = learned.cell_box(cells)
    c = T.Context(M=200, precision=T.PREC_FP32, device=dev)
    c.set_model(m)
    c.density()  # slab-width autotune outside the timings
    l2_flush(dev)
    rz = c.scc_solve()
    l2_flush(dev)
    t = time.perf_counter()
    q_init = learned.warm_start(mlp, m, box)
    t_mlp = time.perf_counter() - t
    c.set_params(mix_beta=learned.MIX_BETA)
    rl = c.scc_solve(q_init=q_init)
    c.close()
    tz, tl = rz["report"]["t_total_ms"] / 1e3, rl["report"]["t_total_ms"] / 1e3 + t_mlp
    out = {"metric": "SCC iterations and s to |dq|<1e-6 e, 8x8x8 cristobalite",
                          "config": {"cells": cells, "atoms": m.natoms, "orbitals": m.n, "sigma_ang": 0.08,
                                     "seed": 8008, "M": 200, "precision": "fp32"},
                          "zero_start": {"iters": rz["iters"], "s": tz},
                          "learned_start": {"iters": rl["iters"], "s": tl, "mlp_s": t_mlp,
                                            "start_err_max_e": float(np.abs(q_init - rz["q"]).max()),
                                            "q0_err_max_e": float(np.abs(m.q0 - rz["q"]).max())},
                          "speedup": tz / tl,
                          "max_dq_between_solutions": float(np.abs(rz["q"] - rl["q"]).max())}
    if rank == 0 and args.learned_eval:
        print(json.dumps(out), flush=True)
    return out


def run_sp2_bench(args, T, dev, rank):
    """SP2 path: 4x4x4 beta-cristobalite (1536 atoms, 6144 orbitals), sigma
    0.08 A, Gershgorin X_0, drop 1e-5 on 4x4 blocks, <= 40 steps."""
    cells = args.cells or [4, 4, 4]
    m = T.model_cristobalite(*cells, sigma_ang=args.sigma_sp2 or 0.08, seed=3003)
    out = {}
    for name, prec in (("fp32", T.PREC_FP32), ("fp64", T.PREC_FP64)):
        c = T.Context(precision=prec, device=dev, sp2_drop_tol=1e-5, sp2_max_iter=40,
                      sp2_idem_tol=1e-10)
        c.set_model(m)
        for _ in range(args.warmup):
            c.sp2()
        ts = []
        for _ in range(args.steps):
            l2_flush(dev)
            r = c.sp2()
            ts.append(r["report"]["t_total_ms"] / 1e3)
        rep = r["report"]
        t = statistics.mean(ts)
        out[name] = {"s_per_solve": t, "iters": rep["sp2_iters"],
                     "gflops": rep["sp2_flops"] / t / 1e9,
                     "gflops_performed": rep["sp2_flops_done"] / t / 1e9,
                     "GBps_algorithmic": rep["sp2_bytes"] / t / 1e9,
                     "idem_err": rep["idem_err"], "nnzb": rep["sp2_nnzb"],
                     "blocks_per_row": rep["sp2_nnzb"] / m.natoms, "e_band": r["e_band"],
                     "q_sum": float(r["q"].sum())}
        out[name + "_q"] = r["q"]
        c.close()
    exact = os.path.join(ROOT, "tests", "golden", "sp2_exact_%dx%dx%d.npz" % tuple(cells))
    if os.path.exists(exact) and args.sigma_sp2 is None:
        ex = np.load(exact)  # dense FP64 eigendecomposition of the same cell
        for name in ("fp32", "fp64"):
            out[name]["vs_exact_projector"] = {
                "max_dq": float(np.abs(out[name + "_q"] - ex["q"]).max()),
                "e_band_per_atom": abs(out[name]["e_band"] - float(ex["e_band"])) / m.natoms}
    dq = float(np.abs(out.pop("fp32_q") - out.pop("fp64_q")).max())
    res = {"metric": "s per SP2 purification (1536 atoms, drop 1e-5)",
                          "config": {"cells": cells, "atoms": m.natoms, "sigma_ang": 0.08,
                                     "seed": 3003, "drop_tol": 1e-5, "max_iter": 40},
                          "fp32": out["fp32"], "fp64": out["fp64"],
                          "max_dq_fp32_vs_fp64": dq}
    if rank == 0 and args.sp2:
        print(json.dumps(res), flush=True)
    return res


def run_all_kernels(T, dev):
    """Every kernel of the library once or a few times on small inputs: the
    program behind the per-kernel launch list (duration and DRAM traffic of
    each kernel under ncu).  Prints one JSON line naming the calls made."""
    from largetb_gb300 import learned
    m = T.model_cristobalite(3, 3, 3, sigma_ang=0.05, seed=7)
    calls = []
    for kern in (T.FP32_STAGED, T.FP32_PERSISTENT, T.FP32_PIPELINED, T.FP32_PIPELINED_STEP):
        with T.Context(M=60, precision=T.PREC_FP32, fp32_kernel=kern, device=dev,
                       column_block=0 if kern == T.FP32_PERSISTENT else 512) as c:
            c.set_model(m)
            c.density()
        calls.append(f"density fp32 kernel {kern}")
    with T.Context(M=60, precision=T.PREC_FP64, scc_max_iter=2, device=dev) as c:
        c.set_model(m)
        c.scc_solve(raise_on_cap=False)
        c.kpm_dos(n_moments=60, n_random=8, seed=1, npts=120)
    calls += ["scc fp64 x2", "kpm_dos"]
    with T.Context(M=60, precision=T.PREC_FP32, check_fp32=1, fp32_kernel=T.FP32_PIPELINED_STEP,
                   column_block=512, scc_max_iter=3, device=dev) as c:
        c.set_model(m)
        c.density()
        c.scc_solve(raise_on_cap=False)
    calls += ["density fp32 + fp64 check", "scc fp32 x3 (graph)"]
    with T.Context(precision=T.PREC_FP32, sp2_max_iter=6, device=dev) as c:
        c.set_model(T.model_cristobalite(2, 2, 2, sigma_ang=0.08, seed=3))
        c.sp2()
    calls.append("sp2 x6")
    with T.Context(M=60, kT=0.0, precision=T.PREC_FP64, device=dev) as c:
        c.set_model(T.model_cristobalite(2, 2, 2, sigma_ang=0.05, seed=5))
        c.density_stochastic(n_probes=16, seed=3, dos_moments=100, dos_points=200)
    calls.append("stochastic density (16 probes)")
    with T.Context(M=60, device=dev) as c:
        c.set_geometry(m.xyz, m.species, learned.cell_box((3, 3, 3)), rcut_bohr=4.0, gamma_diag=1.0)
        c.density()
    calls.append("set_geometry + density")
    for kern in (T.FP32_AUTO, T.FP32_STAGED):
        with T.Batch([T.model_cristobalite(*d, sigma_ang=0.05, seed=i)
                      for i, d in enumerate([(1, 1, 2), (2, 1, 2), (2, 2, 2)])], M=60, device=dev,
                     fp32_kernel=kern) as b:
            b.scc_solve()
        calls.append(f"batch of 3, fp32 kernel {kern}")
    X = T.mlp_features(m.xyz, m.species, learned.cell_box((3, 3, 3)))
    mlp = T.MLP(device=dev, seed=2)
    mlp.train(X, np.zeros(len(X), np.float32), epochs=1, batch=256, lr=1e-3)
    mlp.predict(X)
    mlp.predict_fp32(X)
    calls += ["mlp train 1 epoch", "mlp predict (tensor cores)", "mlp predict fp32"]
    print(json.dumps({"all_kernels": calls}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, nargs=3, default=None)
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 solve (with --batch: the single-structure loops)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the SP2, batch and learned-start figures added to the headline line")
    ap.add_argument("--column-block", type=int, default=0)
    ap.add_argument("--fp32-kernel", type=int, default=0,
                    help="0 autotune, 1 staged, 2 persistent, 3 pipelined (one launch per slab), "
                         "4 pipelined (one launch per step)")
    ap.add_argument("--density-only", action="store_true",
                    help="time single density evaluations (the unit profiled with ncu)")
    ap.add_argument("--zero-start", action="store_true",
                    help="start the timed solves from q0 instead of the learned charges")
    ap.add_argument("--reference-stages", action="store_true",
                    help="the reference's logged stages on its own workload (8x8x8 alpha-quartz)")
    ap.add_argument("--learned-eval", action="store_true",
                    help="8x8x8 cell (12288 atoms): SCC from q0 vs from the learned start (M = 200)")
    ap.add_argument("--batch", action="store_true",
                    help="64 cristobalite cells of random shape solved as one batch (M = 300)")
    ap.add_argument("--structures", type=int, default=64,
                    help="--batch: the first S of the 64 cells (a smaller case for profiling)")
    ap.add_argument("--sp2", action="store_true",
                    help="time SP2 purification of 4x4x4 cristobalite (sigma 0.08 A, drop 1e-5)")
    ap.add_argument("--sigma-sp2", type=float, default=None, help="--sp2: displacement sigma (A)")
    ap.add_argument("--all-kernels", action="store_true",
                    help="run every kernel of the library on small inputs (for the ncu launch list)")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch  # device plumbing only: L2 flush buffer and synchronisation
    import largetb_gb300 as T
    T.load()
    dev = local
    torch.cuda.set_device(dev)
    if args.all_kernels:
        run_all_kernels(T, dev)
        return
    if args.sp2:
        run_sp2_bench(args, T, dev, rank)
        return
    if args.batch:
        run_batch_bench(args, T, dev, rank)
        return
    if args.reference_stages:
        out = run_reference_stages(args, T, dev, rank)
        if rank == 0:
            print(json.dumps(out), flush=True)
        return
    if args.learned_eval:
        run_learned_eval(args, T, dev, rank)
        return
    cells = args.cells or WORKLOAD["cells"]
    cfg = dict(WORKLOAD)
    if args.cells:
        cfg["cells"] = cells
        cfg["workload"] = f"beta-cristobalite {cells[0]}x{cells[1]}x{cells[2]} SCC solve"
    m = T.model_cristobalite(*cells, sigma_ang=cfg["sigma_ang"], seed=cfg["seed"])
    cfg["atoms"], cfg["orbitals"] = m.natoms, m.n
    M = cfg["M"]
    ctx = T.Context(M=M, kT=cfg["kT"], precision=T.PREC_FP32, device=dev,
                    column_block=args.column_block, fp32_kernel=args.fp32_kernel, scc_tol=cfg["scc_tol"])
    ctx.set_model(m)
    if args.density_only:
        for _ in range(args.warmup):
            ctx.density()
        torch.cuda.synchronize(dev)
        ms = []
        for _ in range(args.steps):
            l2_flush(dev)
            rep = ctx.density()["report"]
            ms.append(rep)
        ctx.close()
        if rank == 0:
            tot = sum(r["t_moments_ms"] for r in ms) / 1e3
            b = sum(r["spmm_bytes"] for r in ms)
            nl = sum(r["spmm_launches"] for r in ms)
            print(json.dumps({"metric": "s per density evaluation", "value":
                              statistics.mean(r["t_total_ms"] for r in ms) / 1e3, "unit": "s",
                              "config": cfg, "spmm_launches": nl, "spmm_GBps": b / tot / 1e9,
                              "avg_launch_us": tot * 1e6 / nl, "column_block": ms[-1]["column_block"],
                              "step_kernel": ms[-1]["step_kernel"],
                              "kernel_launches": ms[-1]["kernel_launches"]}), flush=True)
        return

    from largetb_gb300 import learned
    mlp = None if args.zero_start else learned.load(device=dev)
    box = learned.cell_box(cells)
    if mlp is not None:
        ctx.set_params(mix_beta=learned.MIX_BETA)  # the learned start sits close to the fixed point

    def start():
        """Learned starting charges (features + MLP on the GPU) and their wall time."""
        if mlp is None:
            return None, 0.0
        t = time.perf_counter()
        q = learned.warm_start(mlp, m, box)
        return q, time.perf_counter() - t

    for _ in range(args.warmup):
        l2_flush(dev)
        ctx.scc_solve(q_init=start()[0])

    clocks = Clocks(dev)
    barrier(ws)
    torch.cuda.synchronize(dev)
    clocks.start()
    dev_ms, mom_ms, launches, spmm_l, spmm_b, iters = [], [], 0, 0, 0.0, []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        l2_flush(dev)
        q_init, t_start = start()
        r = ctx.scc_solve(q_init=q_init)
        rep = r["report"]
        dev_ms.append(rep["t_total_ms"] + 1e3 * t_start)
        mom_ms.append(rep["t_moments_ms"])
        launches += rep["kernel_launches"] + (2 if mlp is not None else 0)  # + k_features, k_mlp_fb
        spmm_l += rep["spmm_launches"]
        spmm_b += rep["spmm_bytes"]
        iters.append(r["iters"])
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    barrier(ws)
    clk = clocks.stop()
    B = rep["column_block"]
    q32 = r["q"]
    eb32 = r["e_band"]

    # e2e: the public call with host buffers (CSR upload + conversion + solve + readback)
    e2e = []
    h2d = (m.rowptr.nbytes + m.colidx.nbytes + m.vals.nbytes + m.orb2atom.nbytes +
           m.g_rowptr.nbytes + m.g_colidx.nbytes + m.g_vals.nbytes + m.q0.nbytes)
    d2h = m.natoms * 8 + m.n * 8
    barrier(ws)
    for _ in range(args.steps):
        l2_flush(dev)
        t1 = time.perf_counter()
        ctx.set_model(m)
        r2 = ctx.scc_solve(q_init=start()[0])
        e2e.append(time.perf_counter() - t1)
    barrier(ws)
    # the same solve from the neutral charges (the reference's start), default mixer
    ctx.set_params(mix_beta=0.2)
    l2_flush(dev)
    rz = ctx.scc_solve()
    zero = {"s_per_solve": rz["report"]["t_total_ms"] / 1e3, "iters": rz["iters"],
            "max_dq_vs_learned_start": float(np.abs(rz["q"] - q32).max())}

    value = allmax(ws, statistics.mean(dev_ms) / 1e3)
    e2e_v = allmax(ws, statistics.mean(e2e))
    hbm, src = peaks()
    achieved = spmm_b / (sum(mom_ms) / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 recurrence, f64 moments",
        "data": "synthetic (seeded beta-cristobalite)",
        "config": cfg,
        "impl_config": {"column_block": B, "precision": "fp32 recurrence, fp64 moments",
                        "replicas": ws},
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "scc_iterations": iters,
        "start": "learned (MLP, largetb_gb300/data/charge_mlp.npz)" if mlp is not None else "neutral q0",
        "zero_start_fp32": zero,
        "wall_s_per_step": wall / args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm,
                     "traffic": DRAM_TRAFFIC_6X6X6.get((rep["step_kernel"], B)) if list(cells) == [6, 6, 6] else None,
                     "traffic_unit": "DRAM bytes per launch (ncu)", "peak_source": src,
                     "kernel": STEP_KERNELS.get(rep["step_kernel"], "k_cheb_f32"), "launches": int(spmm_l),
                     "avg_launch_us": sum(mom_ms) * 1e3 / max(1, spmm_l),
                     "bytes_per_launch": spmm_b / max(1, spmm_l)},
        "clocks": clk,
    }
    if not args.no_plain:
        ctx64 = T.Context(M=M, kT=cfg["kT"], precision=T.PREC_FP64, device=dev,
                          scc_tol=cfg["scc_tol"])
        ctx64.set_model(m)
        l2_flush(dev)
        r64 = ctx64.scc_solve()
        rep64 = r64["report"]
        q64, eb64 = r64["q"], r64["e_band"]
        line["plain_fp64"] = {"s_per_solve": rep64["t_total_ms"] / 1e3, "iters": r64["iters"],
                              "start": "neutral q0",
                              "moments_s": rep64["t_moments_ms"] / 1e3,
                              "speedup_fast_vs_plain": rep64["t_total_ms"] / 1e3 / value,
                              "max_dq_fast_vs_plain": float(np.abs(q32 - r64["q"]).max()),
                              "e_band_diff_per_atom": abs(eb32 - r64["e_band"]) / m.natoms}
        # the plain form runs M steps per identity column: 32 flop per 4x4 block and column
        nnzb = int(m.rowptr[-1]) // 16
        line["plain_fp64"]["roofline"] = fp64_roofline(
            float(r64["iters"]) * M * nnzb * 32.0 * m.n, rep64["t_moments_ms"] / 1e3, dev)
        # FP32 error alone: both forms on the same H (H0 + Gamma shift of the FP32 charges)
        shift = ctx.coulomb_shift(q32)[m.orb2atom]
        d32, d64 = ctx.density(shift), ctx64.density(shift)
        line["plain_fp64"]["same_H"] = {"max_dq": float(np.abs(d32["q"] - d64["q"]).max()),
                                        "e_band_diff_per_atom": abs(d32["e_band"] - d64["e_band"]) / m.natoms}
        ctx64.close()
    fx = oracle_fixture(cells)
    if fx is not None:
        # against the FP64 oracle's converged SCC of the same cell (fixture)
        line["vs_fp64_oracle"] = {
            "oracle_iters": int(fx["iters"]),
            "fast_max_dq": float(np.abs(q32 - fx["q"]).max()),
            "fast_max_dq_vs_fixed_point": float(np.abs(q32 - fx["q_tight"]).max()),
            "fast_e_band_per_atom": abs(eb32 - float(fx["e_band"])) / m.natoms}
        if "plain_fp64" in line:
            line["vs_fp64_oracle"].update({
                "plain_iters": line["plain_fp64"]["iters"],
                "plain_max_dq": float(np.abs(q64 - fx["q"]).max()),
                "plain_e_band_per_atom": abs(eb64 - float(fx["e_band"])) / m.natoms})
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        O.build()
        mo = O.cristobalite(*cells, sigma_ang=cfg["sigma_ang"], seed=cfg["seed"])
        it = scc_iterations(cells)
        src = "the FP64 oracle's converged SCC of this cell, committed fixture"
        if it is None:
            it = line.get("plain_fp64", {}).get("iters", iters[-1])
            src = "the plain FP64 GPU solve of this cell"
        line["cpu_baseline"] = cpu_sample(mo, M, os.cpu_count() or 1, it, src)
        line["oracle_full_solve_measured"] = measured_oracle_solve(cells)
    ctx.close()
    if not args.no_extras and list(cells) == WORKLOAD["cells"]:
        # the other configurations, measured on the same box after the timed
        # region (outside it): SP2 purification, the 64-cell batch, the
        # learned start on 8x8x8
        sub = argparse.Namespace(**vars(args))
        sub.cells, sub.steps, sub.warmup, sub.no_plain = None, 1, 1, True
        line["sp2_4x4x4"] = run_sp2_bench(sub, T, dev, rank)
        line["batch_64_cells"] = run_batch_bench(sub, T, dev, rank)
        line["learned_start_8x8x8"] = run_learned_eval(sub, T, dev, rank)
        line["reference_logged_stages"] = run_reference_stages(sub, T, dev, rank)
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
