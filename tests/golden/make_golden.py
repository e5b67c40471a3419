"""Convert the reference's own matrix/vector dumps into compact fixtures.

Reads, from a checkout of pghale/largeTB (its path is the first argument), the
PETSc MATLAB-format dumps the reference wrote (MatView/VecView with
PETSC_VIEWER_ASCII_MATLAB) and the Jackson table of runKPM, and writes
tests/golden/reference_dumps.npz:

  amat_{r,c,v}      Amat.m      H of 1x1x1 alpha-quartz (36 x 36)
  h444_{r,c,v}      H.m         H of 4x4x4 alpha-quartz (2304 x 2304)
  gamma_{r,c,v}     GAMMA_AB.m  Gamma of 4x4x4 quartz (576 x 576)
  o2a_{r,c,v}       orbit2Atom.m  orbital -> atom map (576 x 2304)
  dh_{r,c,v}        deltaH.m    delta H of one SCC step (2304 x 2304)
  netcharge         netCharge.m    delta q of that step (576)
  gammaq            GammaQ_vector.m  Gamma * delta q (576)
  gns_col1          gnsfile.txt column 1: Jackson g_n, N = 1000 (6-digit print)
  hscc_{r,c,v}      Htotal_scc.m  H of one SCC iteration (2304 x 2304)
  dosfile           dosfile.txt   runKPM's DOS of Htotal_scc: 2000 x (energy, dos),
                    N = 1000 Jackson moments from 20 Gaussian vectors, printed %lf

Indices are 0-based.  Run once where the reference is mounted; the tests use
only the .npz, never the reference tree.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

_ENTRY = re.compile(r"^\s*(\d+)\s+(\d+)\s+(\S+)\s*$")


def read_mat(path):
    rows, cols, vals = [], [], []
    shape = None
    with open(path) as f:
        for line in f:
            if line.startswith("% Size"):
                a, b = line.split("=")[1].split()
                shape = (int(a), int(b))
            m = _ENTRY.match(line)
            if m:
                rows.append(int(m.group(1)) - 1)
                cols.append(int(m.group(2)) - 1)
                vals.append(float(m.group(3)))
    return (np.array(rows, np.int32), np.array(cols, np.int32), np.array(vals), shape)


def read_vec(path):
    out = []
    with open(path) as f:
        inside = False
        for line in f:
            s = line.strip()
            if s.endswith("= ["):
                inside = True
                continue
            if inside:
                if s.startswith("]"):
                    break
                out.append(float(s))
    return np.array(out)


def main(ref, out=None):
    out = out or os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_dumps.npz")
    d = {}
    for key, name in [("amat", "Amat.m"), ("h444", "H.m"), ("gamma", "GAMMA_AB.m"),
                      ("o2a", "orbit2Atom.m"), ("dh", "deltaH.m"), ("hscc", "Htotal_scc.m")]:
        r, c, v, shape = read_mat(os.path.join(ref, name))
        d[key + "_r"], d[key + "_c"], d[key + "_v"] = r, c, v
        d[key + "_shape"] = np.array(shape, np.int32)
    d["netcharge"] = read_vec(os.path.join(ref, "netCharge.m"))
    d["gammaq"] = read_vec(os.path.join(ref, "GammaQ_vector.m"))
    gns = np.loadtxt(os.path.join(ref, "gnsfile.txt"))
    d["gns_col1"] = gns[:, 0]
    d["dosfile"] = np.loadtxt(os.path.join(ref, "dosfile.txt"), delimiter=",")
    np.savez_compressed(out, **d)
    print("wrote", out, {k: v.shape for k, v in d.items()})


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py REFERENCE_CHECKOUT [OUT.npz]")
    main(*sys.argv[1:])
