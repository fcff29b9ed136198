"""CPU restatement of the reference's collaborative PCS (commit + opening)
for N parties, as the reference's coPCS test runs it with N MPI ranks.

TEST INFRASTRUCTURE ONLY: the checker that the one-device party pipeline
(gbz_pcs_commit / gbz_pcs_open) is compared against, itself pinned to the
transcripts that the unmodified reference wrote when run with N = 4 and 16
ranks (tests/golden/parties_*.json, made by tests/golden/make_golden.py
through oracle/ref's pigeon_mpi).  The product never imports it.

It restates, party by party and then as the leader:
  prepare_parameters  coPCS.cpp:38-72 (get_degrees / get_queries, New_PCS.cpp:23-77)
  prepare_data        coPCS.cpp:76-129
  PCS_commit          coPCS.cpp:236-250  (Encode :131-147, distributed_MT :152-230)
  F_ip                MPI_utils.cpp:483-553 (the opening claim K)
  PCS_open_new        coPCS.cpp:1310-1607, the parties' side and the leader's
                      aggregation: row batching and the first round (:1336-1451),
                      batch_commitments_new (:1242-1308), pcs_sumcheck_phase1/2/3
                      (:547-587, :634-648) with pcs_sumcheck_aggr (MPI_utils.cpp:341-405),
                      encode_concatenated + commit_concatenated (:653-738),
                      delegate_checks' queries, folds and segment gather (:740-891,
                      get_segments MPI_utils.cpp:187-255), RS_multifold5 +
                      commit_tensorcode (:893-919), send_pcs_data (MPI_utils.cpp:58-116)
Small sizes only (Python loops over parties and rounds; the heavy vector
work goes through the C oracle).
"""
import math

import numpy as np

import gbz_oracle as orc

P = orc.P
BATCH_FACTOR = 32      # New_PCS.cpp:10
SECURITY_LEVEL = 100   # New_PCS.cpp:3


# ------------------------------------------------------------------ scalars
def fmul(a, b):
    return ((a[0] * b[0] - a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def fadd(a, b):
    return ((a[0] + b[0]) % P, (a[1] + b[1]) % P)


def fsub(a, b):
    return ((a[0] - b[0]) % P, (a[1] - b[1]) % P)


def fpow(a, e):
    r, x = (1, 0), a
    while e:
        if e & 1:
            r = fmul(r, x)
        x = fmul(x, x)
        e >>= 1
    return r


def finv(a):
    return fpow(a, P * P - 2)


def fe(a):
    return (int(a[0]), int(a[1]))


def arr(values):
    return np.array(values, dtype=np.uint64).reshape(-1, 2)


# ------------------------------------------------------------------ vectors
def vmul(a, b):
    return orc.field_ops(a, b)[2]


def vadd(a, b):
    return orc.field_ops(a, b)[0]


def vsub(a, b):
    return orc.field_ops(a, b)[1]


def vscale(a, s):
    return vmul(a, np.tile(arr([s]), (a.shape[0], 1)))


def vsum(a):
    acc = (0, 0)
    for x in a:
        acc = fadd(acc, fe(x))
    return acc


def vdot(a, b):
    return vsum(vmul(a, b))


def powers(w, n):
    out, x = [], (1, 0)
    for _ in range(n):
        out.append(x)
        x = fmul(x, w)
    return arr(out)


def rou(log_order):
    return fe(orc.root_of_unity(log_order))


def next_pow2(x):
    return 1 << max(0, (x - 1).bit_length())


# ------------------------------------------------------------------ Merkle
G_BLOCK = None


def blake3_words(block64):
    return orc.blake3_64(np.frombuffer(block64, dtype=np.uint8))[0].tobytes()


def leaf_hash(elems4):
    return blake3_words(arr(elems4).tobytes())


def self_hash(h, times):
    for _ in range(times):
        h = blake3_words(h + h)
    return h


def mt_root(elems):
    """Root of MT_commit_Blake (merkle_tree.cpp:195-233) over elems (len >= 4):
    inner nodes hash their left child twice, so the root is leaf 0 hashed
    log2(len / 4) more times."""
    n = elems.shape[0]
    return self_hash(leaf_hash(elems[:4]), int(math.log2(n // 4)))


# ------------------------------------------------------------------ schedule
def schedule(N, M, rates):
    """prepare_parameters (coPCS.cpp:38-72): degrees, queries, rate_offset,
    delegation sizes and the random-share count."""
    rounds = len(rates)
    row_size = 2 * (4 * M // N)
    log_size = int(math.log2(row_size))
    degrees = [BATCH_FACTOR]
    log_size -= int(math.log2(BATCH_FACTOR))
    degrees.append(8)
    log_size -= 3
    deg = int(log_size / (rounds - 2))
    for _ in range(1, rounds - 2):
        degrees.append(1 << deg)
    degrees.append(1 << (log_size - deg * (rounds - 3)))
    queries = []
    for i in range(rounds):
        if i <= 1:
            queries.append(int(SECURITY_LEVEL / (-math.log2(1 - 0.25 * (1.0 - 1.0 / rates[0][0])))))
        else:
            r0, r1 = float(rates[i][0]), float(rates[i][1])
            l1 = int(SECURITY_LEVEL / (-math.log2(1 - 0.5 * 0.5 * (1.0 - 1.0 / r0) * (1 - math.sqrt(1.0 / r1)))))
            l2 = int(SECURITY_LEVEL / (-math.log2(1 - 0.5 * 0.5 * (1.0 - 1.0 / r0))) +
                     SECURITY_LEVEL / (-math.log2(math.sqrt(1.0 / r1))))
            queries.append(l2 if l1 > l2 else l1)
    rate_offset = 1
    for i in range(1, len(rates)):
        rate_offset *= rates[i][0]
    delegation = [next_pow2(degrees[i] * queries[i]) for i in range(2, len(degrees))]
    randomness = sum(q * d for q, d in zip(queries, degrees))
    return dict(N=N, M=M, rates=rates, degrees=degrees, queries=queries, rate_offset=rate_offset,
                delegation=delegation, max_delegation=max(delegation), randomness=randomness)


# ------------------------------------------------------------------ commit
def prepare_data(shares, random, q0):
    """prepare_data (coPCS.cpp:76-129) for one party: the rows of
    Commit_data that have entries (batches of them)."""
    S = shares.shape[0]
    Bs = S // (BATCH_FACTOR // 2)
    rows = []
    dc = rc = 0
    last = None
    for i in range(BATCH_FACTOR):
        row = np.zeros((Bs, 2), dtype=np.uint64)
        for k in range(Bs - q0):
            row[k] = shares[dc]
            dc += 1
            if dc == S:
                break
        for k in range(Bs - q0, Bs):
            row[k] = random[rc]
            rc += 1
        rows.append(row)
        if dc == S:
            last = i
            break
    if dc < S:
        raise ValueError("more batches are needed")
    row = np.zeros((Bs, 2), dtype=np.uint64)
    if S - rc > Bs:
        for k in range(Bs):
            row[k] = random[rc]
            rc += 1
            if rc == random.shape[0]:
                break
    else:
        for k in range(Bs - (S - rc)):
            row[k] = random[rc]
            rc += 1
    rows.append(row)
    assert len(rows) == last + 2
    return np.stack(rows)


def commit(sched, shares, random):
    """PCS_commit for every party: Commit_data rows, codewords (Encode) and
    distributed_MT (column-root tree, its root, the leader's root)."""
    N = sched["N"]
    log_ro = int(math.log2(sched["rate_offset"]))
    parties = []
    for p in range(N):
        cd = prepare_data(shares[p], random[p], sched["queries"][0])
        cw = orc.encode_rows(cd, sched["rates"][0][0], log_ro)
        levels, leader = orc.column_merkle(cw, N)
        parties.append(dict(cd=cd, cw=cw, levels=levels, root=levels[-1].tobytes(), leader=leader.tobytes()))
    return parties


# ------------------------------------------------------------------ opening
def share_map(N):
    """compute_secret_shares' map for one group (MPI_utils.cpp:2747-2762),
    as a function of the _k = N/2 inputs: iFFT, zero-pad to 2N, FFT, odd entries."""
    def apply(x):
        buf = arr(list(x) + [(0, 0)] * (N // 2 - len(x)))
        c = orc.fft(buf, inverse=True)
        c = np.vstack([c, np.zeros((2 * N - N // 2, 2), dtype=np.uint64)])
        ev = orc.fft(c)
        return [fe(ev[2 * j + 1]) for j in range(N)]
    return apply


def unpack_even_sum(cols, N):
    """pcs_sumcheck_aggr's leader step (MPI_utils.cpp:362-371) for one
    coefficient: unpack_secret_share(P, N, N) then the sum of the even entries."""
    sec = arr(cols)
    sec = orc.fft(sec, inverse=True)
    w = finv(rou(1 + int(math.log2(N))))
    sec = vmul(sec, powers(w, N))
    sec = orc.fft(sec)
    acc = (0, 0)
    for j in range(N // 2):
        acc = fadd(acc, fe(sec[2 * j]))
    return acc


def aggregate(polys, N):
    return [unpack_even_sum([fe(polys[p][i]) for p in range(N)], N) for i in range(len(polys[0]))]


def f_ip(parties, sched, r):
    """F_ip (MPI_utils.cpp:483-553) as the coPCS test calls it (main.cpp:87-112)."""
    N = sched["N"]
    lk = int(math.log2(N // 4))
    r2, r1 = r[:lk], r[lk:]
    b1 = orc.precompute_beta(arr(r1))
    b2 = orc.precompute_beta(arr(r2)) if lk else arr([(1, 0)])
    Y = []
    for p in range(N):
        cd = parties[p]["cd"]
        batches = cd.shape[0]
        v = np.zeros((BATCH_FACTOR * cd.shape[1], 2), dtype=np.uint64)
        for i in range(batches - 1):
            v[i::BATCH_FACTOR] = cd[i]
        Y.append(vdot(v, b1[: v.shape[0]]))
    Yv = orc.fft(arr(Y), inverse=True)
    Yv = vmul(Yv, powers(finv(rou(1 + int(math.log2(N)))), N))
    Yv = orc.fft(Yv)
    s = (0, 0)
    for i in range(b2.shape[0]):
        s = fadd(s, fmul(fe(b2[i]), fe(Yv[N * i // (N // 2)])))
    return s


def f_ip_vectors(parties, sched, b1, b2, b3):
    """F_ip (MPI_utils.cpp:483-553) with input vectors as coPIOP_prove forms
    the claim of its PCS opening (the pcs mode of oracle/ref/dpcs_mpi_driver.cpp):
    row weights b1 (32 entries), the row vector b2 with its last _queries[0]
    entries zero (coPCS.cpp:1328-1335), the party weights b3 (N/4 entries)."""
    N = sched["N"]
    b2 = arr(b2).copy()
    q0 = sched["queries"][0]
    b2[len(b2) - q0:] = 0
    b1 = arr(b1)
    Y = []
    for p in range(N):
        cd = parties[p]["cd"]
        batches = cd.shape[0]
        acc = (0, 0)
        for i in range(batches - 1):
            acc = fadd(acc, fmul(fe(b1[i]), fe(vdot(cd[i], b2))))
        Y.append(acc)
    Yv = orc.fft(arr(Y), inverse=True)
    Yv = vmul(Yv, powers(finv(rou(1 + int(math.log2(N)))), N))
    Yv = orc.fft(Yv)
    b3 = arr(b3)
    s = (0, 0)
    for i in range(b3.shape[0]):
        s = fadd(s, fmul(fe(b3[i]), fe(Yv[N * i // (N // 2)])))
    return s


class Chain:
    """Fiat-Shamir prev_challenge (Fiat_Shamir.cpp:5-56)."""

    def __init__(self, state=(0, 0)):
        self.s = arr([state])[0]

    def h2f(self, elems):
        out = orc.hash_to_field(self.s, arr(elems))
        self.s = out
        return fe(out)

    def indexes(self, l, N, M):
        out = []
        for _ in range(l):
            self.s = orc.hash_F(self.s, self.s)
            out.append((int(self.s[0]) % N, int(self.s[1]) % M))
        return out


def party_grouped(qs):
    """The leader's order after get_segments (MPI_utils.cpp:187-255): its own
    queries, then each other party's, each in draw order."""
    return sorted(qs, key=lambda q: q[0])


def phase1(data, B, d):
    """pcs_sumcheck_phase1's local loop (coPCS.cpp:547-566)."""
    poly = [(0, 0)] * (2 * d)
    for j in range(data.shape[0] // d):
        h1 = orc.fft(data[j * d:(j + 1) * d], inverse=True)
        h2 = orc.fft(B[j * d:(j + 1) * d], inverse=True)
        z = np.zeros((d, 2), dtype=np.uint64)
        h1 = orc.fft(np.vstack([h1, z]))
        h2 = orc.fft(np.vstack([h2, z]))
        pr = vmul(h1, h2)
        poly = [fadd(poly[k], fe(pr[k])) for k in range(2 * d)]
    return poly


def fold_blocks(v, L):
    """pcs_sumcheck_phase2's fold (coPCS.cpp:575-586)."""
    return orc.cophase2(v, arr(L))


def open_parties(sched, parties, r, K, fs=(0, 0)):
    """PCS_open_new (coPCS.cpp:1310-1607), parties' side and leader's
    aggregation.  Returns the records the leader sees, in order."""
    N = sched["N"]
    deg, qs, rates = sched["degrees"], sched["queries"], sched["rates"]
    ch = Chain(fs)
    out = dict(polys=[], party_polys=[], challenges=[], K=[], roots=[], queries=[], y=[], segments=[], s=[])
    lk = int(math.log2(N // 4))
    r3 = r[:lk]
    r1 = r[lk:lk + 5]
    Bs = parties[0]["cd"].shape[1]
    r2 = r[lk + 5:lk + 5 + int(math.log2(Bs))]
    b1 = orc.precompute_beta(arr(r1))
    b2 = orc.precompute_beta(arr(r2))
    b3 = orc.precompute_beta(arr(r3)) if lk else arr([(1, 0)])
    batches = parties[0]["cd"].shape[0]
    b1 = [fe(x) for x in b1[:batches]]
    b2 = orc.fft(b2)
    b3p = share_map(N)([fe(x) for x in b3])
    log_ro = int(math.log2(sched["rate_offset"]))
    w = rou(1 + log_ro + int(math.log2(Bs)))
    pw, pwi = powers(w, Bs), powers(finv(w), Bs)
    st = []
    for p in range(N):
        cd, cw = parties[p]["cd"], parties[p]["cw"]
        Cp = np.zeros_like(cw[0])
        bcd = np.zeros_like(cd[0])
        for i in range(batches - 1):
            Cp = vadd(Cp, vscale(cw[i], b1[i]))
            bcd = vadd(bcd, vscale(cd[i], b1[i]))
        bcd = orc.fft(bcd, inverse=True)
        cdl = orc.fft(cd[batches - 1], inverse=True)
        bcd, cdl = vmul(bcd, pwi), vmul(cdl, pwi)
        B = vscale(vmul(b2, pw), b3p[p])
        st.append(dict(Cp=Cp, bcd=bcd, cdl=cdl, B=B, cw_last=cw[batches - 1]))
    # first batching round (coPCS.cpp:1418-1451)
    H = []
    for p in range(N):
        a = vdot(vsub(st[p]["bcd"], st[p]["cdl"]), st[p]["B"])
        b = vdot(st[p]["cdl"], st[p]["B"])
        H.append([a, b, (0, 0)])
    poly = aggregate(H, N)
    out["party_polys"].append(H)
    out["polys"].append(poly)
    if fadd(poly[0], poly[1]) != tuple(K):
        raise AssertionError("first round: the aggregated message does not sum to K")
    rf = ch.h2f(poly)
    out["challenges"].append(rf)
    K = fmul(rf, fadd(poly[1], fmul(rf, poly[0])))
    out["K"].append(K)
    one_m = fsub((1, 0), rf)
    for p in range(N):
        s = st[p]
        s["B"] = vscale(s["B"], rf)
        s["bcd"] = vadd(vscale(s["bcd"], rf), vscale(s["cdl"], one_m))
        s["Cp"] = vadd(vscale(s["Cp"], rf), vscale(s["cw_last"], one_m))
    # batch_commitments_new (coPCS.cpp:1242-1308): column roots of C' with
    # _degrees[1] entries per column, the tree over them, the leader's root
    d1 = deg[1]
    roots = []
    for p in range(N):
        Cp = st[p]["Cp"]
        cols = Cp.shape[0] // d1
        col0 = arr([fe(Cp[k * cols]) for k in range(d1)])
        roots.append(self_hash(mt_root(col0), int(math.log2(cols))))
    out["roots"].append(("batch", roots, self_hash(roots[0], int(math.log2(N)))))
    q = ch.indexes(qs[0], N, parties[0]["cw"].shape[1])
    out["queries"].append(("batch", party_grouped(q)))
    prev_roots, prev_depth = None, -1
    nrounds = len(rates) - 1
    for i in range(nrounds):
        d = deg[i + 1]
        polys = [phase1(st[p]["bcd"], st[p]["B"], d) for p in range(N)]
        poly = aggregate(polys, N)
        out["party_polys"].append(polys)
        out["polys"].append(poly)
        ev = (0, 0)
        for j in range(d):
            ev = fadd(ev, poly[2 * j])
        if ev != tuple(K):
            raise AssertionError("round %d: the aggregated message does not match K" % i)
        c = ch.h2f(poly)
        out["challenges"].append(c)
        L2 = orc.lagrange_coeff(arr([c])[0], int(math.log2(2 * d)))
        K = vdot(arr(poly), L2)
        L = [fe(x) for x in orc.lagrange_coeff(arr([c])[0], int(math.log2(d)))]
        for p in range(N):
            st[p]["bcd"] = fold_blocks(st[p]["bcd"], L)
            st[p]["B"] = fold_blocks(st[p]["B"], L)
        last = i == nrounds - 1
        newC, newCp = [], []
        if not last:
            for p in range(N):
                cpn, cn = orc.encode_concatenated(st[p]["bcd"], rates[i + 2][0], rates[i + 2][1], deg[i + 2])
                newCp.append(cpn)
                newC.append(cn)
            roots = [mt_root(np.asarray(newC[p]).reshape(-1, 2)) for p in range(N)]
            prev_roots = roots
            prev_depth = int(math.log2(np.asarray(newC[0]).reshape(-1, 2).shape[0] // 4))
            out["roots"].append(("concatenated", roots, self_hash(roots[0], int(math.log2(N)))))
        else:
            for p in range(N):
                newCp.append(orc.rs_multifold5(st[p]["Cp"], arr(L)))
            # commit_tensorcode hands MT_commit_Blake the previous commitment's
            # levels; MT_commit_Blake resizes only an empty levels vector
            # (merkle_tree.cpp:205-208), so a shallower tree leaves the old top
            # level in place and the root it reports is the previous root.
            new_depth = int(math.log2(newCp[0].shape[0] // 4))
            if new_depth < prev_depth:
                roots = list(prev_roots)
            else:
                roots = [mt_root(newCp[p]) for p in range(N)]
            out["roots"].append(("tensorcode", roots, self_hash(roots[0], int(math.log2(N)))))
        # delegate_checks (coPCS.cpp:740-891): queries over the segments of
        # the current C', each answered by the RS fold of its segment
        seg_n = st[0]["Cp"].shape[0] // d
        l = qs[i + 1]
        qd = party_grouped(ch.indexes(l, N, seg_n))
        folded = [orc.rs_multifold5(st[p]["Cp"], arr(L)) for p in range(N)]
        y = [fe(folded[a][b]) for a, b in qd]
        segs = [[fe(st[a]["Cp"][b + k * seg_n]) for k in range(d)] for a, b in qd]
        out["queries"].append(("delegate", qd))
        out["y"].append(y)
        out["segments"].append(segs)
        if not last:
            for j, (a, b) in enumerate(qd):
                pos = rates[i + 2][0] * b // rates[i + 1][0]
                if fe(newCp[a][pos]) != y[j]:
                    raise AssertionError("delegate check %d fails" % j)
        for p in range(N):
            st[p]["Cp"] = newCp[p]
        s = ch.h2f([(0, 0)])
        out["s"].append(s)
        if not last:
            qs_scaled = [(a, rates[i + 2][0] * b // rates[i + 1][0]) for a, b in qd]
            for p in range(N):
                st[p]["B"] = orc.pcs_phase3(st[p]["B"], qs_scaled, arr([s])[0], N, rates[i + 2][0], p)
            pk = s
            for j in range(len(y)):
                K = fadd(K, fmul(pk, y[j]))
                pk = fmul(pk, s)
        out["K"].append(K)
    out["final"] = [(st[p]["bcd"], st[p]["B"], st[p]["Cp"]) for p in range(N)]
    out["fs"] = fe(ch.s)
    return out
