"""FP64-oracle SCC fixture for the 6x6x6 beta-cristobalite solve.

Runs the CPU oracle's exact-trace SCC (oracle/tb_oracle.c: orc_density +
orc_anderson in orc_scc's order, the working form of the SCC loop of
withSP2_deltaH.cpp:1820-1840) on the cell the headline solve uses:

  6x6x6 beta-cristobalite (5184 atoms, 20736 orbitals), a = 7.16 A,
  sigma = 0.05 A, seed 2002, 4-bohr cutoff, Gamma diagonal +1 Ha,
  KPE M = 400, Jackson damping, kT = 0.01 Ha, Anderson history 16,
  beta 0.2, start from the neutral charges q0.

It records the state at the first iteration whose residual
max_a |q_out - q_in| is below 1e-6 e (what orc_scc(tol = 1e-6) returns:
charges, band energy, mu, iteration count) and then continues the same
Anderson run until the residual is below 1e-8 e, which gives the fixed point
itself to ~1e-8 e.  A few sums of the model's arrays are stored so a test can
confirm that it rebuilt the same Hamiltonian.

One density evaluation is ~40 TFLOP of FP64 block products (about 250 s on
8 x86 cores), so the whole run takes a few hours on the CPU.  After every
iteration the loop state (iterate, mixer ring, history) is written to a
checkpoint file; a run started again with the same arguments continues from
it, with iterates bit-identical to an uninterrupted run.  Usage:

  python tests/golden/make_scc_oracle.py [nx ny nz] [--threads N] [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def model_sums(rowptr, vals, xyz):
    """Order-independent fingerprints of a model (H values and positions)."""
    return np.array([len(rowptr) - 1, rowptr[-1], float(np.sum(vals)), float(np.sum(vals * vals)),
                     float(np.sum(np.abs(vals))), float(np.sum(xyz))])


def _save_ckpt(path, loop, hist, t_eval, snap):
    tmp = path + ".tmp.npz"
    extra = {} if snap is None else {f"snap_{k}": np.asarray(v) for k, v in snap.items()}
    np.savez(tmp, hist=np.array(hist), t_eval=np.array(t_eval), **loop.state(), **extra)
    os.replace(tmp, path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cells", type=int, nargs="*", default=[6, 6, 6])
    ap.add_argument("--M", type=int, default=400)
    ap.add_argument("--seed", type=int, default=2002)
    ap.add_argument("--sigma", type=float, default=0.05)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--tight", type=float, default=1e-8)
    ap.add_argument("--max-iter", type=int, default=60)
    ap.add_argument("--out", default=None)
    ap.add_argument("--checkpoint", default=None,
                    help="loop-state file (default: <out> with .ckpt.npz)")
    args = ap.parse_args()
    from oracle import oracle as O
    O.build()
    nx, ny, nz = args.cells
    out = args.out or os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                   f"scc_oracle_{nx}x{ny}x{nz}.npz")
    ckpt = args.checkpoint or out[:-4] + ".ckpt.npz"
    m = O.cristobalite(nx, ny, nz, sigma_ang=args.sigma, seed=args.seed)
    p = O.kpe_params(M=args.M, kT=0.01, n_elec=m.n_elec, nthreads=args.threads)
    loop = O.SccLoop(m, p, beta=0.2, history=16)
    snap, hist, t_eval = None, [], []
    if os.path.exists(ckpt):
        c = np.load(ckpt)
        loop.restore(c)
        hist, t_eval = list(c["hist"]), list(c["t_eval"])
        if "snap_iters" in c.files:
            snap = {k[5:]: (c[k] if c[k].ndim else c[k].item()) for k in c.files
                    if k.startswith("snap_")}
        print("resuming after iteration", loop.it, flush=True)
    t0 = time.perf_counter()
    while True:
        t1 = time.perf_counter()
        it, q_in, r, mx = loop.step()
        t_eval.append(time.perf_counter() - t1)
        hist.append(mx)
        print(json.dumps({"iter": it, "dq_max": mx, "s": round(t_eval[-1], 1),
                          "e_band": r["e_band"], "mu": r["mu"]}), flush=True)
        if snap is None and mx < 1e-6:
            snap = dict(iters=it, q=r["q"].copy(), e_band=r["e_band"], mu=r["mu"], a=r["a"],
                        b=r["b"], q_in=q_in.copy())
        if mx < args.tight or it >= args.max_iter or not mx < 1e3:
            break
        _save_ckpt(ckpt, loop, hist, t_eval, snap)
    if snap is None:
        raise SystemExit(f"no convergence to 1e-6 e in {it} iterations")
    np.savez_compressed(
        out, cells=np.array(args.cells, np.int32), M=args.M, seed=args.seed, sigma_ang=args.sigma,
        kT=0.01, beta=0.2, history=16, tol=1e-6,
        iters=snap["iters"], q=snap["q"], e_band=snap["e_band"], mu=snap["mu"], a=snap["a"],
        b=snap["b"],
        tight_tol=args.tight, tight_iters=it, q_tight=r["q"], e_band_tight=r["e_band"],
        mu_tight=r["mu"], dq_hist=np.array(hist), eval_s=np.array(t_eval),
        threads=args.threads or (os.cpu_count() or 1),
        model_sums=model_sums(m.rowptr, m.val, m.xyz))
    print("wrote", out, "iterations to 1e-6:", snap["iters"], "to", args.tight, ":", it,
          "total s:", round(time.perf_counter() - t0, 1))


if __name__ == "__main__":
    main()
