"""Exact density matrix for the SP2 workload, by dense eigendecomposition.

The SP2 purification (withSP2.cpp:956-1044: getSP2/computeAlphas) converges
to the zero-temperature projector onto the N_e/2 lowest eigenstates of H;
dropping 4x4 blocks below the drop tolerance truncates it.  This script
builds the 4x4x4 beta-cristobalite cell the SP2 path is measured on (1536
atoms, 6144 orbitals, sigma 0.08 A, seed 3003, reference block model, 4-bohr
cutoff) with the oracle's builder, diagonalises H in FP64 (LAPACK through
numpy) and stores

  q       Mulliken charges 2 sum_{i in a} P_ii (electrons, both spins)
  e_band  2 sum of the occupied eigenvalues (Ha)
  n_occ   occupied states (N_e / 2), homo, lumo (Ha)

so the tests can state the truncation error of the thresholded block SP2
against the exact projector.  Usage:

  python tests/golden/make_sp2_exact.py [nx ny nz] [--out PATH]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cells", type=int, nargs="*", default=[4, 4, 4])
    ap.add_argument("--sigma", type=float, default=0.08)
    ap.add_argument("--seed", type=int, default=3003)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    import scipy.sparse as sp
    from oracle import oracle as O
    O.build()
    nx, ny, nz = args.cells
    out = args.out or os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                   f"sp2_exact_{nx}x{ny}x{nz}.npz")
    m = O.cristobalite(nx, ny, nz, sigma_ang=args.sigma, seed=args.seed)
    H = sp.csr_matrix((m.val, m.col, m.rowptr), shape=(m.n, m.n)).toarray()
    H = (H + H.T) / 2
    n_occ = int(round(m.n_elec / 2))
    w, V = np.linalg.eigh(H)
    Vo = V[:, :n_occ]
    diagP = np.einsum("ij,ij->i", Vo, Vo)
    q = 2 * np.bincount(m.orb2atom, diagP, minlength=m.natoms)
    np.savez_compressed(out, cells=np.array(args.cells, np.int32), sigma_ang=args.sigma,
                        seed=args.seed, q=q, e_band=2 * w[:n_occ].sum(), n_occ=n_occ,
                        homo=w[n_occ - 1], lumo=w[n_occ], lmin=w[0], lmax=w[-1])
    print("wrote", out, "gap (Ha):", w[n_occ] - w[n_occ - 1], "E_band:", 2 * w[:n_occ].sum())


if __name__ == "__main__":
    main()
