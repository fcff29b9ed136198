"""CPU restatement of the reference's distributed PCS commitments for N
parties (Batch_dCommit and dCommit, distributed_PCS.cpp:56-170).

TEST INFRASTRUCTURE ONLY: the checker that gbz_dpcs_batch_commit /
gbz_dpcs_commit are compared against, itself pinned to what the unmodified
reference computed with N ranks (tests/golden/dpcs.json, written through
oracle/ref's pigeon_dpcs by tests/golden/make_golden.py).  The product never
imports it.

The reference's distributed FFT (distributed_batch_FFT / distributed_FFT,
MPI_utils.cpp:2911-3298: a local transform on every rank, an all-to-all and
N-point butterflies across the ranks) is one transform of length N L of the
message interleaved across the parties (party p's entry t is coefficient
t N + p); party r keeps, for every m < N, the L/N outputs starting at
r L/N + m L.  Each party's tree hashes columns of its codeword rows
(MT_commit_Blake over the column) and builds create_tree_blake over them.
"""
import numpy as np

import gbz_oracle as orc


def codewords(arrs, rows, rate):
    """Batch rows of every party's codeword: arrs N x A; row k of party p is
    arrs[p][k S:(k+1) S] zero-padded to L = rate S; returns N x rows x L."""
    N, A = arrs.shape[0], arrs.shape[1]
    S = A // rows
    L = S * rate
    out = np.zeros((N, rows, L, 2), dtype=np.uint64)
    blk = L // N
    for k in range(rows):
        G = np.zeros((N * L, 2), dtype=np.uint64)
        for p in range(N):
            G[p:N * S:N] = arrs[p, k * S:(k + 1) * S]
        X = orc.fft(G)
        for r in range(N):
            out[r, k] = np.concatenate([X[r * blk + m * L:r * blk + m * L + blk] for m in range(N)])
    return out


def column_hashes(rows):
    """MT_commit_Blake's root over every column of rows (nrows x len): the
    leaf of the column's first four entries, then a self-hash per level
    above it (merkle_tree.cpp:201-221, 267-299)."""
    nrows, n = rows.shape[0], rows.shape[1]
    out = np.zeros((n, 32), dtype=np.uint8)
    for j in range(n):
        out[j] = orc.merkle_commit(np.ascontiguousarray(rows[:, j]))[-1]
    return out


def tree_levels(leaves):
    """create_tree_blake over leaf hashes (merkle_tree.cpp:267-300): node i
    of a level is blake3(child 2i || child 2i); every level, leaves first,
    as one (2 n - 1) x 32 array."""
    levels = [np.ascontiguousarray(leaves, dtype=np.uint8)]
    while levels[-1].shape[0] > 1:
        left = levels[-1][0::2]
        levels.append(orc.blake3_64(np.concatenate([left, left], axis=1)))
    return np.concatenate(levels)


def commit(arrs, rows, rate, column_height=None):
    """Every party's codeword rows and tree: Batch_dCommit (rows batch rows,
    columns over the rows) or, with column_height, dCommit (one row, columns
    of column_height entries spaced L / column_height apart).  Returns
    (codewords N x rows x L, levels per party, roots)."""
    cw = codewords(arrs, rows, rate)
    lv = []
    for p in range(arrs.shape[0]):
        grid = cw[p] if column_height is None else cw[p, 0].reshape(column_height, -1, 2)
        lv.append(tree_levels(column_hashes(grid)))
    return cw, lv, [x[-1] for x in lv]
