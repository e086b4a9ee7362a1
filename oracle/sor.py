"""Oracle restatement of the multicolour order of the SOR / SSOR sweeps (test
infrastructure only).

The reference's TMatrix::sor_sweep (src/Matrix/Matrix.C:943-1031) visits the
rows in their natural order. The GPU sweep runs colour by colour: a greedy
colouring of the matrix graph (rows i and j adjacent when a_ij or a_ji is
stored), in row order, each row taking the smallest colour none of its
already coloured neighbours has. Rows of one colour do not couple, so their
updates are independent, and the colour-by-colour sweep equals the sequential
sweep over the rows ordered by colour (increasing row number within a colour).
orc_sor_sweep in oracle.c runs that sequential sweep for a given order.
"""
from __future__ import annotations

import numpy as np


def greedy_colouring(row_ptr: np.ndarray, cols: np.ndarray) -> np.ndarray:
    """colour of every row (int32)"""
    n = row_ptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(row_ptr))
    keep = rows != cols
    a, b = rows[keep], cols[keep]
    # symmetric adjacency in CSR form
    src = np.concatenate([a, b])
    dst = np.concatenate([b, a])
    o = np.lexsort((dst, src))
    src, dst = src[o], dst[o]
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ptr, src + 1, 1)
    ptr = np.cumsum(ptr)
    colour = np.full(n, -1, dtype=np.int32)
    for i in range(n):
        nb = dst[ptr[i]:ptr[i + 1]]
        used = colour[nb[nb < i]]
        c = 0
        if used.size:
            taken = np.zeros(used.max() + 2, dtype=bool)
            taken[used] = True
            c = int(np.argmin(taken))
        colour[i] = c
    return colour


def colour_order(colour: np.ndarray) -> np.ndarray:
    """rows grouped by colour, increasing row number within a colour (int32)"""
    return np.lexsort((np.arange(colour.size), colour)).astype(np.int32)
