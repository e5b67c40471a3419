"""PETSc ASCII MATLAB dumps <-> CSR arrays.

The reference writes its matrices and vectors with
``PetscViewerPushFormat(viewer, PETSC_VIEWER_ASCII_MATLAB)`` (e.g. the H, Gamma
and delta-H dumps of withSP2_deltaH.cpp:948-965, 1464-1485, 1503-1523): a
``% Size = m n`` header and 1-based ``i j value`` triplets for a Mat, one value
per line between ``= [`` and ``];`` for a Vec.  ``read_mat`` turns such a dump
into sorted CSR arrays ready for ``tb_set_hamiltonian`` / ``tb_set_scc``;
``write_mat`` / ``write_vec`` produce the same format.
"""
from __future__ import annotations

import re

import numpy as np

_TRIPLET = re.compile(r"^\s*(\d+)\s+(\d+)\s+(\S+)\s*$")


def read_mat(path):
    """Return (rowptr, colidx, vals, (m, n)) of a MATLAB-format PETSc Mat dump.

    Entries keep their stored order per row after a stable sort by column;
    duplicated (i, j) entries are summed."""
    rows, cols, vals = [], [], []
    shape = None
    with open(path) as f:
        for line in f:
            if line.startswith("% Size"):
                a, b = line.split("=")[1].split()
                shape = (int(a), int(b))
                continue
            m = _TRIPLET.match(line)
            if m:
                rows.append(int(m.group(1)) - 1)
                cols.append(int(m.group(2)) - 1)
                vals.append(float(m.group(3)))
    if shape is None:
        raise ValueError(f"{path}: no '% Size' header (not a PETSc MATLAB Mat dump)")
    return coo_to_csr(np.array(rows, np.int64), np.array(cols, np.int64), np.array(vals), shape)


def coo_to_csr(r, c, v, shape):
    m, _ = shape
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    if len(r):
        key = r * (shape[1] + 1) + c
        uniq, first = np.unique(key, return_index=True)
        v = np.add.reduceat(v, first)
        r, c = r[first], c[first]
    rowptr = np.zeros(m + 1, np.int64)
    np.add.at(rowptr, r + 1, 1)
    return (np.cumsum(rowptr).astype(np.int32), c.astype(np.int32), v.astype(np.float64), shape)


def read_vec(path):
    out, inside = [], False
    with open(path) as f:
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


def write_mat(path, rowptr, colidx, vals, shape, name="zzz"):
    nnz = int(rowptr[-1])
    with open(path, "w") as f:
        f.write("%Mat Object: 1 MPI processes\n%  type: seqaij\n")
        f.write(f"% Size = {shape[0]} {shape[1]} \n% Nonzeros = {nnz} \n")
        f.write(f"{name} = zeros({nnz},3);\n{name} = [\n")
        for i in range(shape[0]):
            for k in range(rowptr[i], rowptr[i + 1]):
                f.write(f"{i + 1} {colidx[k] + 1}  {vals[k]:.16e}\n")
        f.write(f"];\n")


def write_vec(path, v, name="Vec_0"):
    with open(path, "w") as f:
        f.write(f"%Vec Object: 1 MPI processes\n%  type: seq\n{name} = [\n")
        for x in v:
            f.write(f"{x:.16e}\n")
        f.write("];\n")
