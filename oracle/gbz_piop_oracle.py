"""CPU restatement of the reference's R1CS front end up to its second
sumcheck (`pigeon 1`: coPIOP_prove, coPIOP.cpp:1382-1648) for N parties.

TEST INFRASTRUCTURE ONLY: it regenerates the parties' inputs of prove_phase1
and prove_phase2 exactly as rank 0 deals them, and restates the data steps
of the two phases, so that the one-device implementation (gbz_piop_phase1 /
gbz_piop_phase2) can be compared with what the unmodified reference computed
when run with N = 8 and 16 ranks (tests/golden/piop_*.json, written by
tests/golden/make_golden.py through oracle/ref's pigeon_mpi).  The product
never imports it.

Dealing (rank 0, glibc generator seeded by srand(42) inside the circuit
generator):
  generate_R1CS_matrixes, type 1   coPIOP.cpp:95-193 (add_input, add_mul)
  transpose_R1CS_matrixes          coPIOP.cpp:61-93
  distribute_index's row split     MPI_utils.cpp:2483-2597, parse_R1CS_matrixes :2205-2270
  prepare_witness_data, type 1     utils.cpp:1363-1424
  distribute_proving_data          MPI_utils.cpp:2813-2866
  generate_sumcheck_randomness     MPI_utils.cpp:3633-3700
  setup_randomness                 MPI_utils.cpp:2868-2900
Data steps of the phases:
  _beta, y and its interpolation   coPIOP.cpp:241-300
  compute_Kr / sum                 MPI_utils.cpp:3620-3631, 3370-3414
  _reduce_R1CS_matrixes_multivariate  Distributed_Sumcheck.cpp:2283-2350
  secret_share_vector              Distributed_Sumcheck.cpp:2352-2400
  compute_beta_shares_multivariate coPIOP.cpp:348-379
  the witness layout after PCS_commit  coPIOP.cpp:1550-1563
Between its own draws, the reference's rank 0 makes others (the sparse
evaluation index); the caller passes where the generator stood when
distribute_proving_data began (the fixture's record of it), and the rest
follows from the draws restated here.
"""
import math

import numpy as np

import gbz_oracle as orc

P = orc.P
SEED = 42              # coPIOP.cpp:164


def _log2(x):
    return x.bit_length() - 1


def next_pow2(x):
    return 1 << max(0, (x - 1).bit_length())


# --------------------------------------------------------------- the circuit
def circuit(M):
    """generate_R1CS_matrixes(M, 1): M/16 input gates, then for each of the
    remaining M - M/16 steps a coin rand() % 2 that either adds one more
    left wire to the next multiplication gate or closes it (add_mul: its
    left wires drawn rand() % gates without repeats, its right wire
    rand() % gates).  Returns the gates' left wire lists and right wires,
    logm, logn and the draws it made."""
    g = orc.Prng(SEED)
    n_in = M // 16
    draws = [0]

    def rnd():
        draws[0] += 1
        return g.next()

    lefts, rights = [], []
    count = n_in

    def add_mul(size, add_ctr):
        wires = [rnd() % size]
        for _ in range(add_ctr - 1):
            while True:
                num = rnd() % size
                if num not in wires:
                    wires.append(num)
                    break
        lefts.append(wires)
        rights.append(rnd() % size)

    add_ctr = 0
    for _ in range(n_in, M):
        if rnd() % 2 == 0:
            add_ctr += 1
        else:
            add_mul(count, add_ctr)
            count += 1
            add_ctr = 0
    if add_ctr != 0:
        add_mul(count, add_ctr)
        count += 1
    muls = len(lefts)
    return {"M": M, "inputs": n_in, "lefts": lefts, "rights": rights,
            "logm": _log2(next_pow2(muls)), "logn": _log2(next_pow2(n_in + muls)), "draws": draws[0]}


def r1cs_rows(c, N):
    """The transposed matrices split over N parties (what pA, pB, pC hold on
    each rank): per matrix, per party, CSR arrays (row_ptr over the party's
    2^logn / N rows, then cols).  Entries of a row keep the order of
    transpose_R1CS_matrixes (by constraint, then by wire)."""
    n_in = c["inputs"]
    rows = 1 << c["logn"]
    per = rows // N
    entries = {
        "A": ([w for l in c["lefts"] for w in l],
              [t for t, l in enumerate(c["lefts"]) for _ in l]),
        "B": (list(c["rights"]), list(range(len(c["rights"])))),
        "C": ([n_in + t for t in range(len(c["lefts"]))], list(range(len(c["lefts"])))),
    }
    out = {}
    for name, (r, col) in entries.items():
        r = np.asarray(r, dtype=np.int64)
        col = np.asarray(col, dtype=np.int64)
        order = np.argsort(r, kind="stable")
        r, col = r[order], col[order]
        ptr = np.searchsorted(r, np.arange(rows + 1), side="left")
        parts = []
        for p in range(N):
            a, b = ptr[p * per], ptr[(p + 1) * per]
            parts.append((ptr[p * per:(p + 1) * per + 1] - a, col[a:b].copy()))
        out[name] = parts
    return out


def witness_data(c, g):
    """prepare_witness_data(M, W, L, R, O, 1): the inputs drawn by
    generate_randomness(M/16), then every gate in order: L = sum of its left
    wires, R = its right wire, O = L·R appended to the witness.  All values
    lie in the base field.  W padded to 2^logn, L, R, O to 2^logm."""
    W = [int(x) for x in orc.generate_randomness(g, c["inputs"])[:, 0]]
    L, R, O = [], [], []
    for left, right in zip(c["lefts"], c["rights"]):
        s = sum(W[w] for w in left) % P
        r = W[right]
        o = s * r % P
        L.append(s)
        R.append(r)
        O.append(o)
        W.append(o)
    W += [0] * ((1 << c["logn"]) - len(W))
    m = 1 << c["logm"]
    for v in (L, R, O):
        v += [0] * (m - len(v))
    base = lambda v: np.stack([np.asarray(v, dtype=np.uint64), np.zeros(len(v), dtype=np.uint64)], axis=1)
    return base(W), base(L), base(R), base(O)


def phase_degrees(n_vl, n_w):
    """degrees1 from the parties' vL length and degrees2 from their witness
    share length (coPIOP.cpp:1410-1421)."""
    lv = _log2(n_vl)
    d2 = (lv - 4) // 2
    d3 = (lv - 4) - d2
    lw = _log2(2 * n_w) - 5
    e1 = lw // 2
    return [16, 1 << d2, 1 << d3, 2], [1 << e1, 1 << (lw - e1), 32]


def sumcheck_randomness(g, N, degrees1, degrees2):
    """generate_sumcheck_randomness: per degree and per secret slot j < N/4
    a vector of generate_randomness(4 d) (first phase) or (2 d) (second
    phase); K = the sum of the even entries of the second phase's; each
    degree's N/4 vectors transposed, flattened and shared.  Returns per
    party the flattened shares of both phases, and K."""
    k = N // 4
    R1 = [[orc.generate_randomness(g, 4 * d) for _ in range(k)] for d in degrees1]
    R2 = [[orc.generate_randomness(g, 2 * d) for _ in range(k)] for d in degrees2]
    K = 0
    for vs in R2:
        for v in vs:
            K = (K + int(v[0::2, 0].astype(object).sum())) % P
    assert all(int(v[:, 1].max(initial=0)) == 0 for vs in R2 for v in vs)

    def deal(R):
        out = []
        for vs in R:
            temp = np.stack(vs, axis=1).reshape(-1, 2)      # transpose(R[i]) flattened
            out.append(orc.secret_shares_from(temp, N, g))
        return np.concatenate(out, axis=1)
    return deal(R1), deal(R2), K


def setup_randomness(g, N, size):
    """setup_randomness(R, N, N/2, N/4, size): N/4 · size values random(),
    shared: size entries per party."""
    k = N // 4
    vals = np.zeros((k * size, 2), dtype=np.uint64)
    for i in range(k * size):
        vals[i, 0] = g.next()
    return orc.secret_shares_from(vals, N, g)


def deal(N, M, draws_before, pcs_randomness, mask_l):
    """Rank 0's dealing for pigeon 1 with N parties and circuit size M:
    draws_before = the generator's draws since srand(42) when
    distribute_proving_data began; pcs_randomness = the PCS masking length
    per party (prepare_parameters); the mask randomness R has mask_l + 13
    entries per party."""
    c = circuit(M)
    assert c["draws"] <= draws_before
    g = orc.Prng(SEED)
    g.skip(draws_before)
    counts = {"proving_data": draws_before}
    W, L, R, O = witness_data(c, g)
    drawn = draws_before + c["inputs"] + (c["inputs"] + 99) // 100
    shares = {}
    for name, v in (("W", W), ("L", L), ("R", R), ("O", O)):
        shares[name] = orc.secret_shares_from(v, N, g)
        drawn += (v.shape[0] // (N // 4)) * (N // 2 - N // 4)
    counts["sumcheck_randomness"] = drawn
    degrees1, degrees2 = phase_degrees(shares["L"].shape[1], shares["W"].shape[1])
    R1, R2, K = sumcheck_randomness(g, N, degrees1, degrees2)
    return {"circuit": c, "W": shares["W"], "vL": shares["L"], "vR": shares["R"], "vO": shares["O"],
            "degrees1": degrees1, "degrees2": degrees2, "R1": R1, "R2": R2, "K": K,
            "pcs_random": setup_randomness(g, N, pcs_randomness),
            "R": setup_randomness(g, N, mask_l + 13), "counts": counts}


# ------------------------------------------------------------- phase steps
def lagrange(r, d):
    """compute_lagrange_coeff(getRootOfUnity(log2 d), r, d) (utils.cpp)."""
    return orc.lagrange_coeff(r, _log2(d))


def tensor(vectors):
    """buff[j + k·|acc|] = L[k]·acc[j], folded left to right (the products of
    compute_beta_shares_multivariate and _reduce_R1CS_matrixes_multivariate)."""
    acc = vectors[0]
    for L in vectors[1:]:
        acc = np.concatenate([orc.field_ops(acc, np.repeat(L[k:k + 1], acc.shape[0], axis=0))[2]
                              for k in range(L.shape[0])])
    return acc


def r1cs_reduce(parts, r, degrees1, logm, N):
    """_reduce_R1CS_matrixes_multivariate on every party: degrees' = (N/4,
    degrees1 without its last); beta1 = the tensor of the Lagrange vectors
    of degrees'[0..2] at r[0..2], beta2 = the Lagrange vector of degrees'[3]
    at r[3]; row j of party p: sum over its entries (row, col) of
    beta1[col mod S]·beta2[col div S], S = 2^logm / |beta2|."""
    d = [N // 4] + list(degrees1[:-1])
    beta1 = tensor([lagrange(r[i], d[i]) for i in range(len(d) - 1)])
    beta2 = lagrange(r[len(r) - 1], d[len(r) - 1])
    S = (1 << logm) // beta2.shape[0]
    out = []
    for ptr, cols in parts:
        vals = orc.field_ops(beta1[cols % S], beta2[cols // S])[2]
        acc = np.zeros((ptr.shape[0] - 1, 2), dtype=np.uint64)
        for j in range(acc.shape[0]):
            a, b = ptr[j], ptr[j + 1]
            s = [0, 0]
            for t in range(a, b):
                s[0] = (s[0] + int(vals[t, 0])) % P
                s[1] = (s[1] + int(vals[t, 1])) % P
            acc[j] = s
        out.append(acc)
    return np.stack(out)


def share_map(N):
    """The packed-sharing matrix: share p of a group (v_0..v_{k-1}, 0..0)
    is sum_j mu[p][j]·v_j (zero-padded inverse transform of length N/2,
    forward transform of length 2N, entry 2p + 1)."""
    k, kk = N // 4, N // 2
    mu = np.zeros((N, k, 2), dtype=np.uint64)
    for j in range(k):
        buf = np.zeros((kk, 2), dtype=np.uint64)
        buf[j, 0] = 1
        buf = orc.fft(buf, inverse=True)
        ext = np.zeros((2 * N, 2), dtype=np.uint64)
        ext[:kk] = buf
        ext = orc.fft(ext)
        for p in range(N):
            mu[p, j] = ext[2 * p + 1]
    return mu


def reshare(v, N):
    """secret_share_vector on every party: party q shares its vector in
    groups of N/4 with zero padding (no draws); party p receives the shares
    numbered p of every party, party by party: N·|v|/(N/4) entries."""
    k = N // 4
    mu = share_map(N)
    n = v.shape[1]
    out = np.zeros((N, N * (n // k), 2), dtype=np.uint64)
    for q in range(N):
        groups = v[q].reshape(n // k, k, 2)
        for p in range(N):
            acc = np.zeros((n // k, 2), dtype=np.uint64)
            for j in range(k):
                prod = orc.field_ops(groups[:, j], np.repeat(mu[p, j:j + 1], n // k, axis=0))[2]
                acc = orc.field_ops(acc, prod)[0]
            out[p, q * (n // k):(q + 1) * (n // k)] = acc
    return out


def share_scalars(vec, N):
    """b[2p + 1] of compute_beta_shares_multivariate: the first N/4 entries
    of vec zero-padded to N/2, inverse transform, zero-padded to 2N, forward
    transform; entry 2p + 1 for every party p."""
    kk = N // 2
    buf = np.zeros((kk, 2), dtype=np.uint64)
    buf[:vec.shape[0]] = vec
    buf = orc.fft(buf, inverse=True)
    ext = np.zeros((2 * N, 2), dtype=np.uint64)
    ext[:kk] = buf
    ext = orc.fft(ext)
    return ext[1::2].copy()


def witness_layout(commit_rows, row_len, mask_l):
    """The witness prove_phase2 receives (coPCS commit data put back,
    coPIOP.cpp:1550-1563): PCS_commit has cleared the share vector
    (coPCS.cpp:248), so it is rows × row_len zeros; for each non-empty
    commit row but the last, its first row_len - mask_l entries are written
    at row · row_len; then padded to a power of two."""
    rows = len(commit_rows)
    w = np.zeros((rows * row_len, 2), dtype=np.uint64)
    batches = 0
    for r in commit_rows:
        if r.shape[0] == 0:
            break
        batches += 1
    for i in range(batches - 1):
        w[i * row_len:i * row_len + row_len - mask_l] = commit_rows[i][:row_len - mask_l]
    total = w.shape[0]
    if total & (total - 1):
        w = np.concatenate([w, np.zeros((next_pow2(total) - total, 2), dtype=np.uint64)])
    return w


def fs_draws(fs, count):
    """count draws hash_to_field({0}) from the chain state fs."""
    out = []
    for _ in range(count):
        fs = orc.hash_to_field(fs, np.zeros((1, 2), dtype=np.uint64))
        out.append(fs.copy())
    return np.array(out, dtype=np.uint64).reshape(-1, 2), fs


def beta_index(i, r):
    """_beta(i, r) (utils.cpp:1323-1335): prod_t (bit t of i ? r_t : 1 - r_t)."""
    one = np.array([[1, 0]], dtype=np.uint64)
    acc = one.copy()
    for t in range(r.shape[0]):
        f = r[t:t + 1] if (i >> t) & 1 else orc.field_ops(one, r[t:t + 1])[1]
        acc = orc.field_ops(acc, f)[2]
    return acc[0]


def unpack_even_dot(shares, b):
    """sum_{i < N/4} b[i] · unpack_secret_share(shares, N, N)[2 i]
    (MPI_utils.cpp:2769-2785 with the leader's sums of sum /
    sumcheck_aggr): the shares interpolated at the odd points of the 2N-th
    roots of unity and read at the even ones."""
    N = shares.shape[0]
    x = orc.fft(shares, inverse=True)
    w = orc.field_ops(np.repeat(orc.root_of_unity(1 + _log2(N)).reshape(1, 2), 1, axis=0),
                      np.zeros((1, 2), dtype=np.uint64))[4]          # inverse of the 2N-th root
    pw = np.zeros((N, 2), dtype=np.uint64)
    pw[0] = [1, 0]
    for i in range(1, N):
        pw[i] = orc.field_ops(pw[i - 1:i], w)[2][0]
    x = orc.fft(orc.field_ops(x, pw)[2])
    acc = np.zeros((1, 2), dtype=np.uint64)
    for i in range(b.shape[0]):
        acc = orc.field_ops(acc, orc.field_ops(b[i:i + 1], x[2 * i:2 * i + 1])[2])[0]
    return acc[0]


def extend(v, mask):
    """A party's vector zero-extended to twice its length with its four
    mask entries at the start of the new half (coPIOP.cpp:289-298)."""
    n = v.shape[0]
    out = np.zeros((2 * n, 2), dtype=np.uint64)
    out[:n] = v
    out[n:n + mask.shape[0]] = mask
    return out


def ip_vector(challenges, degrees, step):
    """The coSumcheck's ip_vec flattened (coSumcheck.cpp:240-275, 345-381):
    round i's entry j = L_i[j] · prod_{t != i} L_t[0], L_t = the Lagrange
    vector over step · d_t points at round t's challenge."""
    Ls = [lagrange(challenges[t], step * d) for t, d in enumerate(degrees)]
    out = []
    for i, L in enumerate(Ls):
        v = L.copy()
        for t, Lt in enumerate(Ls):
            if t != i:
                v = orc.field_ops(v, np.repeat(Lt[0:1], v.shape[0], axis=0))[2]
        out.append(v)
    return np.concatenate(out)


def scale(v, s):
    return orc.field_ops(v, np.repeat(np.asarray(s, dtype=np.uint64).reshape(1, 2), v.shape[0], axis=0))[2]


def segment_aggr(v, mask_l):
    """prove_phase2's 32 segments of 2|v|/32 entries, each holding the next
    2|v|/32 - mask_l entries of v then zeros (coPIOP.cpp:470-488)."""
    seg = 2 * v.shape[0] // 32
    out = np.zeros((32, seg, 2), dtype=np.uint64)
    ctr = 0
    for i in range(32):
        take = min(seg - mask_l, v.shape[0] - ctr)
        out[i, :take] = v[ctr:ctr + take]
        ctr += take
        if ctr == v.shape[0]:
            break
    return out.reshape(-1, 2)
