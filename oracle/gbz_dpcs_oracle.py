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


# ------------------------------------------------------------------ opening
def _h2f(fs, elems):
    """hash_to_field(elems) from the chain state fs (which is left as it
    was): the new state, a copy."""
    st = np.array(fs, dtype=np.uint64, copy=True)
    return orc.hash_to_field(st, elems).copy()


def _sum(v):
    acc = np.zeros((1, 2), dtype=np.uint64)
    for x in v:
        acc = orc.field_ops(acc, x.reshape(1, 2))[0]
    return acc[0]


def _scale(v, s):
    return orc.field_ops(v, np.repeat(np.asarray(s, dtype=np.uint64).reshape(1, 2), v.shape[0], axis=0))[2]


def _add(a, b):
    return orc.field_ops(a, b)[0]


def fold_degrees(N):
    """prepare_data's fold degrees after the batch size (distributed_PCS.cpp:28-54)."""
    lN = N.bit_length() - 1
    d = [1 << (lN - lN // 2)]
    if (1 << (lN // 2)) > 1:
        d.append(1 << (lN // 2))
    return d


def query_draws(fs, l, N, M):
    """get_indexes (Fiat_Shamir.cpp:37-53): l steps prev = hash_F(prev, prev),
    (party, position) = (real mod N, img mod M)."""
    out = []
    for _ in range(l):
        fs = orc.hash_F(fs, fs).copy()
        out.append((int(fs[0]) % N, int(fs[1]) % M))
    return fs, out


def party_blocks(X, N, L, D):
    """Party r's slice of a global codeword X of length N L / D held in the
    distributed layout: for m < N / D the L/N entries from r L/N + m L."""
    seg = L // N
    return [np.concatenate([X[r * seg + m * L:r * seg + m * L + seg] for m in range(N // D)]) for r in range(N)]


def open_batch(cd, cw_global, L, r, y, N, rate, queries_l, verify=(True, False)):
    """PIOP_dOpen_batch_new (distributed_PCS.cpp:1175-1534) of N parties with
    batches = 1, from the Fiat-Shamir state 0.  cd[l][p]: party p's rows of
    polynomial l (rows x S); cw_global[l]: the polynomial's codeword rows as
    one global array per row (rows x N L, natural order); r[l], y[l]: its
    point and claim.  Returns a dict of everything the protocol exposes."""
    P = len(cd)
    rows, S = cd[0][0].shape[0], cd[0][0].shape[1]
    lS, lR, lN = S.bit_length() - 1, (rows - 1).bit_length(), N.bit_length() - 1
    fs = np.zeros(2, dtype=np.uint64)
    b1, b2, b3 = [], [], []
    for l in range(P):
        b2.append(orc.precompute_beta(r[l][:lS]))
        b3.append(orc.precompute_beta(r[l][lS:lS + lR]))
        b1.append(orc.precompute_beta(r[l][lS + lR:lS + lR + lN]))
    # row batching of every party's data and of the global codewords
    cdb = [[_sum_rows(cd[l][p], b3[l]) for p in range(N)] for l in range(P)]
    cwb = [_sum_rows(cw_global[l], b3[l]) for l in range(P)]
    # eval claims: for i, j != i: sum_k b2_j[k] cd'_i[k] b1_j[p], summed over the parties
    K = [[np.zeros(2, dtype=np.uint64) for _ in range(P - 1)] for _ in range(P)]
    for i in range(P):
        t = 0
        for j in range(P):
            if j == i:
                continue
            for p in range(N):
                v = orc.field_ops(_dot_vec(b2[j], cdb[i][p]).reshape(1, 2), b1[j][p:p + 1])[2][0]
                K[i][t] = orc.field_ops(K[i][t].reshape(1, 2), v.reshape(1, 2))[0][0]
            t += 1
    flatK = np.array([x for row in K for x in row], dtype=np.uint64).reshape(-1, 2)
    a0 = _h2f(fs, flatK)
    a1 = _h2f(a0, np.zeros((1, 2), dtype=np.uint64))
    fs = a1
    b = []
    for _ in range(2):
        fs = _h2f(fs, np.zeros((1, 2), dtype=np.uint64))
        b.append(fs)
    b[0] = np.zeros(2, dtype=np.uint64)
    m = lambda u, v: orc.field_ops(u.reshape(1, 2), v.reshape(1, 2))[2][0]
    ad = lambda u, v: orc.field_ops(u.reshape(1, 2), v.reshape(1, 2))[0][0]
    if P == 3:
        y0 = ad(ad(ad(y[0], m(a0, K[0][0])), m(a1, K[0][1])),
                ad(m(b[0], ad(ad(K[1][0], m(a0, y[1])), m(a1, K[1][1]))),
                   m(b[1], ad(ad(K[2][0], m(a0, K[2][1])), m(a1, y[2])))))
    else:
        y0 = ad(ad(y[0], m(a0, K[0][0])), m(b[0], ad(K[1][0], m(a0, y[1]))))
    # PIOP_dBatch_batched_new's weights {1, a[0], a[1]} are, at its call
    # (distributed_PCS.cpp:1291), the vector b = {0, b1}: the data and the
    # codeword of polynomial l > 0 enter with weight b[l - 1]
    Bw = [np.array([1, 0], dtype=np.uint64), b[0], b[1]]
    arr = [np.zeros((S, 2), dtype=np.uint64) for _ in range(N)]
    for p in range(N):
        for l in range(P):
            arr[p] = _add(arr[p], _scale(cdb[l][p], Bw[l]))
    cw = np.zeros((N * L, 2), dtype=np.uint64)
    for l in range(P):
        cw = _add(cw, _scale(cwb[l], Bw[l]))
    degs = fold_degrees(N)
    out = {"K": flatK, "a": [a0, a1], "b1": b[1], "y0": y0, "roots": [], "leader_roots": [], "queries": [],
           "polys": [], "challenges": [], "flags": 0}
    # the batched codeword's commitment: columns of d1 entries spaced |cw_p| / d1
    fs = _commit_round(out, cw, N, L, 1, degs[0], fs, queries_l, M=L)
    # the betas: b2_0 b1_0[p] + a0 b2_1 b1_1[p] (+ a1 b2_2 b1_2[p]) (:1293-1301)
    Aw = [np.array([1, 0], dtype=np.uint64), a0, a1]
    Bv = []
    for p in range(N):
        v = _scale(b2[0], b1[0][p])
        for l in range(1, P):
            v = _add(v, _scale(_scale(b2[l], Aw[l]), b1[l][p]))
        Bv.append(v)
    Kc = y0
    D = 1
    for i, d in enumerate(degs):
        poly = np.zeros((2 * d, 2), dtype=np.uint64)
        for p in range(N):
            poly = _add(poly, _block_products(arr[p], Bv[p], d))
        ev = _sum(poly[0::2])
        if not np.array_equal(ev, Kc) and verify[0]:
            out["flags"] |= 1
            return out
        fs = _h2f(fs, poly)
        c = fs
        out["polys"].append(poly)
        out["challenges"].append(c)
        L2 = orc.lagrange_coeff(c, (2 * d).bit_length() - 1)
        Kc = _sum(orc.field_ops(poly, L2)[2])
        Ld = orc.lagrange_coeff(c, d.bit_length() - 1)
        arr = [_fold(a, Ld, d) for a in arr]
        Bv = [_fold(v, Ld, d) for v in Bv]
        cw = orc.rs_multifold5(cw, Ld)
        D *= d
        if i < len(degs) - 1:
            fs = _commit_round(out, cw, N, L, D, d, fs, queries_l)
    out["arr"] = np.concatenate(arr)
    out["B"] = np.concatenate(Bv)
    out["codeword"] = cw
    out["K_final"] = Kc
    out["fs"] = fs
    return out


def _sum_rows(rows, w):
    acc = np.zeros_like(rows[0])
    for h in range(rows.shape[0]):
        acc = _add(acc, _scale(rows[h], w[h]))
    return acc


def _dot_vec(a, b):
    return _sum(orc.field_ops(a, b)[2])


def _block_products(a, bvec, d):
    """distributed_pcs_sumcheck_phase1_batch's local sum
    (distributed_PCS.cpp:515-541): per block of d entries, the two blocks
    inverse-transformed, zero-padded to 2d, transformed, multiplied."""
    out = np.zeros((2 * d, 2), dtype=np.uint64)
    for j in range(a.shape[0] // d):
        h1 = np.zeros((2 * d, 2), dtype=np.uint64)
        h2 = np.zeros((2 * d, 2), dtype=np.uint64)
        h1[:d] = orc.fft(a[j * d:(j + 1) * d], inverse=True)
        h2[:d] = orc.fft(bvec[j * d:(j + 1) * d], inverse=True)
        out = _add(out, orc.field_ops(orc.fft(h1), orc.fft(h2))[2])
    return out


def _fold(v, Ld, d):
    """distributed_pcs_sumcheck_phase2's fold (distributed_PCS.cpp:546-562)."""
    blocks = v.reshape(-1, d, 2)
    out = np.zeros((blocks.shape[0], 2), dtype=np.uint64)
    for k in range(d):
        out = _add(out, _scale(blocks[:, k], Ld[k]))
    return out


def _commit_round(out, cw, N, L, D, d, fs, queries_l, M=None):
    """Every party's commitment of its slice of the global codeword cw
    (columns of d entries spaced |slice| / d, their trees, the roots) and
    the get_indexes draws that follow (distributed_PCS.cpp:340-360,
    612-680)."""
    slices = party_blocks(cw, N, L, D)
    roots = []
    for sl in slices:
        lv = tree_levels(column_hashes(sl.reshape(d, -1, 2)))
        roots.append(lv[-1])
    out["roots"].append(roots)
    # distributed_commit_batch builds the leader's tree over N zero hashes,
    # whatever the parties' roots (coPCS.cpp:398-408)
    lead = np.zeros((1, 32), dtype=np.uint8)
    for _ in range(N.bit_length() - 1):
        lead = orc.blake3_64(np.concatenate([lead, lead], axis=1))
    out["leader_roots"].append(lead[0])
    # the batched commitment draws positions of the whole slice
    # (:359), a FRI commitment positions of its columns (:661)
    M = slices[0].shape[0] // d if M is None else M
    fs, q = query_draws(fs, queries_l, N, M)
    out.setdefault("query_ranges", []).append(M)
    out["queries"].append(q)
    return fs
