"""ctypes binding for the CPU oracle (oracle/gbz_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The product never imports it.

Field elements travel as numpy uint64 arrays of shape (n, 2): column 0 is
`real`, column 1 is `img` (virgo::fieldElement layout).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgbz_oracle.so")
SRC = os.path.join(HERE, "gbz_oracle.c")

P = (1 << 61) - 1


def build(force=False):
    """Compile the oracle with gcc (portable C11 + pthreads; x86-64 and Arm)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run(["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", "-o", tmp, SRC, "-lpthread", "-lm"],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


class _Prng(ctypes.Structure):
    _fields_ = [("tbl", ctypes.c_int32 * 31), ("f", ctypes.c_int), ("r", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        u64p = ctypes.POINTER(ctypes.c_uint64)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        i64 = ctypes.c_int64
        L.orc_prng_next.restype = ctypes.c_int32
        L.orc_prng_skip.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.orc_merkle_commit.restype = ctypes.c_int
        L.orc_merkle_open.restype = ctypes.c_int
        L.orc_whir_queries.restype = ctypes.c_int
        L.orc_transcript_bytes.restype = i64
        L.orc_transcript_bytes.argtypes = [ctypes.c_int, ctypes.c_int]
        L.orc_prove.restype = i64
        L.orc_prove.argtypes = [u64p, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, u8p, i64, ctypes.c_int]
        L.orc_fft.argtypes = [u64p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_merkle_commit.argtypes = [u64p, i64, u8p, ctypes.c_int]
        L.orc_merkle_open.argtypes = [u8p, i64, i64, u8p]
        L.orc_witness.argtypes = [ctypes.c_uint64, i64, u64p]
        _lib = L
    return _lib


def _p64(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


def _p8(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def fe_array(n):
    return np.zeros((n, 2), dtype=np.uint64)


def witness(seed, n):
    out = fe_array(n)
    lib().orc_witness(ctypes.c_uint64(seed), n, _p64(out))
    return out


def field_ops(a, b):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    n = a.shape[0]
    outs = [fe_array(n) for _ in range(5)]
    lib().orc_field_ops(ctypes.c_int64(n), _p64(a), _p64(b), *[_p64(o) for o in outs])
    return outs  # add, sub, mul, neg, inv


def root_of_unity(log_order):
    out = np.zeros(2, dtype=np.uint64)
    lib().orc_root_of_unity(log_order, _p64(out))
    return out


def blake3_64(blocks):
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 64)
    out = np.zeros((blocks.shape[0], 32), dtype=np.uint8)
    lib().orc_blake3_64(ctypes.c_int64(blocks.shape[0]), _p8(blocks), _p8(out))
    return out


def fft(a, inverse=False, threads=0):
    a = np.array(a, dtype=np.uint64, copy=True).reshape(-1, 2)
    logn = int(a.shape[0]).bit_length() - 1
    lib().orc_fft(_p64(a), logn, int(inverse), threads)
    return a


def merkle_commit(elems, threads=0):
    elems = np.ascontiguousarray(elems, dtype=np.uint64).reshape(-1, 2)
    N = elems.shape[0]
    out = np.zeros((max(N // 2 - 1, 1), 32), dtype=np.uint8)
    rc = lib().orc_merkle_commit(_p64(elems), N, _p8(out), threads)
    if rc != 0:
        raise ValueError("merkle_commit needs a power-of-two length >= 4")
    return out


def merkle_open(levels, N, pos):
    levels = np.ascontiguousarray(levels, dtype=np.uint8)
    depth = (N // 4).bit_length() - 1
    out = np.zeros((max(depth, 1), 32), dtype=np.uint8)
    d = lib().orc_merkle_open(_p8(levels), N, pos, _p8(out))
    if d < 0:
        raise ValueError("position out of range")
    return out[:d]


def hash_F(x, y):
    x = np.ascontiguousarray(x, dtype=np.uint64)
    y = np.ascontiguousarray(y, dtype=np.uint64)
    out = np.zeros(2, dtype=np.uint64)
    lib().orc_hash_F(_p64(x), _p64(y), _p64(out))
    return out


def hash_to_field(state, elems):
    elems = np.ascontiguousarray(elems, dtype=np.uint64).reshape(-1, 2)
    out = np.zeros(2, dtype=np.uint64)
    lib().orc_hash_to_field(_p64(state), _p64(elems), ctypes.c_int(elems.shape[0]), _p64(out))
    return out


class Prng:
    """glibc random()/rand() replica; F::_random via field()."""

    def __init__(self, seed=1):
        self.s = _Prng()
        lib().orc_prng_seed(ctypes.byref(self.s), ctypes.c_uint32(seed))

    def next(self):
        return lib().orc_prng_next(ctypes.byref(self.s))

    def skip(self, count):
        """Drops count random() outputs."""
        lib().orc_prng_skip(ctypes.byref(self.s), count)

    def state(self):
        """The 33 words of the generator (table, front and rear index)."""
        return bytes(self.s)

    @classmethod
    def from_state(cls, state):
        g = cls(1)
        ctypes.memmove(ctypes.addressof(g.s), state, ctypes.sizeof(g.s))
        return g

    def field(self):
        out = np.zeros(2, dtype=np.uint64)
        lib().orc_prng_field(ctypes.byref(self.s), _p64(out))
        return out


def precompute_beta(r, threads=0):
    r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
    out = fe_array(1 << r.shape[0])
    lib().orc_precompute_beta(_p64(r), ctypes.c_int(r.shape[0]), _p64(out), ctypes.c_int(threads))
    return out


def evaluate_vector(v, r):
    v = np.ascontiguousarray(v, dtype=np.uint64).reshape(-1, 2)
    r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
    out = np.zeros(2, dtype=np.uint64)
    lib().orc_evaluate_vector(_p64(v), ctypes.c_int64(v.shape[0]), _p64(r), _p64(out))
    return out


def beta_identity(r1, r2):
    r1 = np.ascontiguousarray(r1, dtype=np.uint64).reshape(-1, 2)
    r2 = np.ascontiguousarray(r2, dtype=np.uint64).reshape(-1, 2)
    out = np.zeros(2, dtype=np.uint64)
    lib().orc_beta_identity(_p64(r1), _p64(r2), ctypes.c_int(r1.shape[0]), _p64(out))
    return out


def sumcheck_quadratic(v1, v2, threads=0):
    v1 = np.ascontiguousarray(v1, dtype=np.uint64).reshape(-1, 2)
    v2 = np.ascontiguousarray(v2, dtype=np.uint64).reshape(-1, 2)
    out = np.zeros(6, dtype=np.uint64)
    lib().orc_sumcheck_quadratic(_p64(v1), _p64(v2), ctypes.c_int64(v1.shape[0]), _p64(out),
                                 ctypes.c_int(threads))
    return out.reshape(3, 2)


def sumcheck_fold(v, r, threads=0):
    v = np.array(v, dtype=np.uint64, copy=True).reshape(-1, 2)
    r = np.ascontiguousarray(r, dtype=np.uint64)
    lib().orc_sumcheck_fold(_p64(v), ctypes.c_int64(v.shape[0]), _p64(r), ctypes.c_int(threads))
    return v[: v.shape[0] // 2].copy()


def rs_fold_tensor(segment, r, n, idx):
    segment = np.ascontiguousarray(segment, dtype=np.uint64).reshape(-1, 2)
    r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
    logk = segment.shape[0].bit_length() - 1
    out = np.zeros(2, dtype=np.uint64)
    lib().orc_rs_fold_tensor(_p64(segment), ctypes.c_int(logk), _p64(r), ctypes.c_int64(n),
                             ctypes.c_int64(idx), _p64(out))
    return out


def rs_multifold5(codeword, a, threads=0):
    codeword = np.ascontiguousarray(codeword, dtype=np.uint64).reshape(-1, 2)
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2)
    logd = a.shape[0].bit_length() - 1
    out = fe_array(codeword.shape[0] >> logd)
    lib().orc_rs_multifold5(_p64(codeword), ctypes.c_int64(codeword.shape[0]), _p64(a), ctypes.c_int(logd),
                            _p64(out), ctypes.c_int(threads))
    return out


def update_betas(b, queries, N, r, threads=0):
    b = np.array(b, dtype=np.uint64, copy=True).reshape(-1, 2)
    q = np.ascontiguousarray(queries, dtype=np.int32)
    r = np.ascontiguousarray(r, dtype=np.uint64)
    ch = fe_array(len(q))
    lib().orc_update_betas(_p64(b), ctypes.c_int64(b.shape[0]), q.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                           ctypes.c_int(len(q)), ctypes.c_int64(N), _p64(r), _p64(ch), ctypes.c_int(threads))
    return b, ch


def whir_queries(rate):
    return lib().orc_whir_queries(ctypes.c_int(rate))


def transcript_bytes(logn, rate):
    return lib().orc_transcript_bytes(logn, rate)


def prove(w, logn, rate, prng_seed=1, threads=0):
    w = np.ascontiguousarray(w, dtype=np.uint64).reshape(-1, 2)
    assert w.shape[0] == 1 << logn
    cap = transcript_bytes(logn, rate)
    out = np.zeros(cap, dtype=np.uint8)
    n = lib().orc_prove(_p64(w), logn, rate, prng_seed, _p8(out), cap, threads)
    if n < 0:
        raise ValueError("oracle prove failed")
    return out[:n].tobytes()


# ---------------------------------------------------------------- coPCS side

def lagrange_coeff(r, logd):
    r = np.ascontiguousarray(r, dtype=np.uint64)
    out = fe_array(1 << logd)
    lib().orc_lagrange_coeff(_p64(r), ctypes.c_int(logd), _p64(out))
    return out


def encode_rows(rows, rate, log_rate_offset, threads=0):
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    nrows, n = rows.shape[0], rows.shape[1]
    logrow = n.bit_length() - 1
    out = np.zeros((nrows, n * rate, 2), dtype=np.uint64)
    lib().orc_encode_rows(_p64(rows), ctypes.c_int(nrows), ctypes.c_int(logrow), ctypes.c_int(rate),
                          ctypes.c_int(log_rate_offset), _p64(out), ctypes.c_int(threads))
    return out


def column_merkle(rows, N):
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    nrows, L = rows.shape[0], rows.shape[1]
    levels = np.zeros((2 * L - 1, 32), dtype=np.uint8)
    root = np.zeros(32, dtype=np.uint8)
    lib().orc_column_merkle(_p64(rows), ctypes.c_int(nrows), ctypes.c_int(L.bit_length() - 1), ctypes.c_int(N),
                            _p8(levels), _p8(root))
    return levels, root


def secret_shares(v, N, privacy=False, prng_seed=1):
    v = np.ascontiguousarray(v, dtype=np.uint64).reshape(-1, 2)
    M = v.shape[0]
    out = np.zeros((N, M // (N // 4), 2), dtype=np.uint64)
    lib().orc_secret_shares(_p64(v), ctypes.c_int64(M), ctypes.c_int(N), ctypes.c_int(int(privacy)),
                            ctypes.c_uint32(prng_seed), _p64(out))
    return out


def generate_randomness(g, n):
    """generate_randomness (utils.cpp:1285-1295) drawing from the Prng g:
    c = random() every 100 entries, entry = c + rand()."""
    out = fe_array(n)
    lib().orc_generate_randomness(ctypes.byref(g.s), ctypes.c_int64(n), _p64(out))
    return out


def secret_shares_from(v, N, g, privacy=True):
    """compute_secret_shares(v, ·, N, N/4, N/2, privacy) (MPI_utils.cpp:2738-2766),
    the privacy entries drawn from the Prng g: N x len(v)/(N/4) shares."""
    v = np.ascontiguousarray(v, dtype=np.uint64).reshape(-1, 2)
    M = v.shape[0]
    out = np.zeros((N, M // (N // 4), 2), dtype=np.uint64)
    lib().orc_secret_shares_g(_p64(v), ctypes.c_int64(M), ctypes.c_int(N), ctypes.c_int(int(privacy)),
                              ctypes.byref(g.s), _p64(out))
    return out


def copcs_party_shares(N, M, R, state=False):
    """Party shares of the reference's coPCS test (main.cpp:49-68) at N
    parties: (shares N x 4M/N, random N x 4R/N), rank 0's glibc draws; with
    state, also the generator's 33 words as the dealing leaves them."""
    k = N // 4
    sh = np.zeros((N, M // k, 2), dtype=np.uint64)
    rn = np.zeros((N, R // k, 2), dtype=np.uint64)
    g = _Prng()
    lib().orc_copcs_party_shares_g(ctypes.c_int(N), ctypes.c_int64(M), ctypes.c_int64(R), _p64(sh), _p64(rn),
                                   ctypes.byref(g))
    return (sh, rn, bytes(g)) if state else (sh, rn)


def party_aggregate(msgs, b):
    msgs = np.ascontiguousarray(msgs, dtype=np.uint64)
    N, length = msgs.shape[0], msgs.shape[1]
    b = np.ascontiguousarray(b, dtype=np.uint64).reshape(-1, 2)
    out = fe_array(length)
    lib().orc_party_aggregate(_p64(msgs), ctypes.c_int(N), ctypes.c_int64(length), _p64(b), _p64(out))
    return out


def cophase1(p1, p2, p3, b1, logd):
    arrs = [np.ascontiguousarray(x, dtype=np.uint64).reshape(-1, 2) for x in (p1, p2, p3, b1)]
    d = 1 << logd
    H, H4 = fe_array(2 * d), fe_array(4 * d)
    lib().orc_cophase1(*[_p64(a) for a in arrs], ctypes.c_int64(arrs[0].shape[0]), ctypes.c_int(logd), _p64(H),
                       _p64(H4))
    return H, H4


def cophase2(v, L):
    v = np.ascontiguousarray(v, dtype=np.uint64).reshape(-1, 2)
    L = np.ascontiguousarray(L, dtype=np.uint64).reshape(-1, 2)
    logd = L.shape[0].bit_length() - 1
    out = fe_array(v.shape[0] // L.shape[0])
    lib().orc_cophase2(_p64(v), ctypes.c_int64(v.shape[0]), _p64(L), ctypes.c_int(logd), _p64(out))
    return out


FORM_VECTORS = {0: 2, 1: 3, 2: 6, 3: 6, 4: 4}
FORM_DEGREE = {0: 2, 1: 3, 2: 2, 3: 3, 4: 4}


def sumcheck_round(form, vecs, b=None):
    """Round message of a sumcheck form over the pairs of vecs (see gbz_oracle.h)."""
    vs = [np.ascontiguousarray(v, dtype=np.uint64).reshape(-1, 2) for v in vecs]
    assert len(vs) == FORM_VECTORS[form]
    arr = (ctypes.c_void_p * len(vs))(*[v.ctypes.data for v in vs])
    out = fe_array(FORM_DEGREE[form] + 1)
    bb = None if b is None else np.ascontiguousarray(b, dtype=np.uint64).reshape(2)
    lib().orc_sumcheck_round(ctypes.c_int(form), arr, ctypes.c_int64(vs[0].shape[0]),
                             None if bb is None else _p64(bb), _p64(out))
    return out


def sumcheck_fold_many(vecs, r):
    """Folded copies (first halves) of every vector."""
    vs = [np.array(np.asarray(v, dtype=np.uint64).reshape(-1, 2), copy=True) for v in vecs]
    arr = (ctypes.c_void_p * len(vs))(*[v.ctypes.data for v in vs])
    rr = np.ascontiguousarray(r, dtype=np.uint64).reshape(2)
    lib().orc_sumcheck_fold_many(ctypes.c_int(len(vs)), arr, ctypes.c_int64(vs[0].shape[0]), _p64(rr))
    return [v[: v.shape[0] // 2].copy() for v in vs]


def party_sumcheck(form, vecs, N, w=None, offset=4, fs=(0, 0), prng_seed=1, y=None):
    """_quadratic_sumcheck (form 0) / _cubic_sumcheck (form 1) of N parties
    (vectors of N*M entries, party-major).  Returns a dict with y (final
    claim), polys, challenges, fin (leader's v[0] values) and fs (chain)."""
    nv = FORM_VECTORS[form]
    vs = [np.array(np.asarray(v, dtype=np.uint64).reshape(-1, 2), copy=True) for v in vecs]
    assert len(vs) == nv
    M = vs[0].shape[0] // N
    lm = M.bit_length() - 1
    rounds = max(lm - offset, 0)
    S = (1 << offset) if rounds > 0 else M
    nchal = rounds + (S * N).bit_length() - 1
    nc = FORM_DEGREE[form] + 1
    polys = fe_array(nc * max(nchal, 1))
    chal = fe_array(max(nchal, 1))
    fin = fe_array(nv)
    w = np.ascontiguousarray(w if w is not None else np.tile([1, 0], (N, 1)), dtype=np.uint64).reshape(-1, 2)
    fsa = np.ascontiguousarray(fs, dtype=np.uint64).reshape(2).copy()
    ya = np.ascontiguousarray(y if y is not None else [0, 0], dtype=np.uint64).reshape(2).copy()
    g = Prng(prng_seed)
    v3 = vs[2] if nv == 3 else None
    lib().orc_party_sumcheck(ctypes.c_int(form), _p64(vs[0]), _p64(vs[1]), None if v3 is None else _p64(v3),
                             ctypes.c_int64(M), ctypes.c_int(N), _p64(w), ctypes.c_int(offset), _p64(fsa),
                             ctypes.byref(g.s), _p64(ya), _p64(polys), _p64(chal), _p64(fin))
    return {"y": ya, "polys": polys[: nc * nchal].reshape(nchal, nc, 2), "challenges": chal[:nchal], "fin": fin,
            "fs": fsa, "prng": g}


def _ptr_array(vs):
    return (ctypes.c_void_p * max(len(vs), 1))(*[v.ctypes.data for v in vs])


def aggregate_claims(arrays, points, prng_seed=1, prng=None):
    """aggregate_claims (Whir.cpp:608-668).  Returns arr, b_aggr, K,
    challenges (c beta then k array challenges), sums (k x c)."""
    arrs = [np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2) for a in arrays]
    pts = np.ascontiguousarray(points, dtype=np.uint64).reshape(len(points), -1, 2)
    k, n, c = len(arrs), arrs[0].shape[0], pts.shape[0]
    arr, b, K = fe_array(n), fe_array(n), np.zeros(2, dtype=np.uint64)
    chal, sums = fe_array(c + k), fe_array(max(k * c, 1))
    g = prng if prng is not None else Prng(prng_seed)
    lib().orc_aggregate_claims(ctypes.c_int(k), _ptr_array(arrs), ctypes.c_int64(n), ctypes.c_int(c), _p64(pts),
                               ctypes.byref(g.s), _p64(arr), _p64(b), _p64(K), _p64(chal), _p64(sums))
    return arr, b, K, chal, sums[: k * c].reshape(k, c, 2)


def aggregate_arrays(arr, b, arrays, B, r1, r2):
    """aggregate_arrays (Whir.cpp:670-704): returns (arr', b', K)."""
    arr = np.array(np.asarray(arr, dtype=np.uint64).reshape(-1, 2), copy=True)
    b = np.array(np.asarray(b, dtype=np.uint64).reshape(-1, 2), copy=True)
    arrs = [np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2) for a in arrays]
    Bs = [np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2) for a in B]
    r1 = np.ascontiguousarray(r1, dtype=np.uint64).reshape(-1, 2)
    r2 = np.ascontiguousarray(r2, dtype=np.uint64).reshape(-1, 2)
    K = np.zeros(2, dtype=np.uint64)
    lib().orc_aggregate_arrays(_p64(arr), _p64(b), ctypes.c_int(len(arrs)), _ptr_array(arrs), ctypes.c_int(len(Bs)),
                               _ptr_array(Bs), ctypes.c_int64(arr.shape[0]), _p64(r1), _p64(r2), _p64(K))
    return arr, b, K


def aggregate_commitments(codewords, r, rate, whir_k=4, prng_seed=1, prng=None):
    """aggregate_commitments (Whir.cpp:547-606): (codeword, levels, prng)."""
    cws = [np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2) for a in codewords]
    n = cws[0].shape[0]
    r = np.ascontiguousarray(r, dtype=np.uint64).reshape(-1, 2)
    cw = fe_array(n)
    leaves = n // whir_k
    levels = np.zeros((2 * leaves - 1, 32), dtype=np.uint8)
    g = prng if prng is not None else Prng(prng_seed)
    lib().orc_aggregate_commitments(ctypes.c_int(len(cws)), _ptr_array(cws), ctypes.c_int64(n), _p64(r),
                                    ctypes.c_int(rate), ctypes.c_int(whir_k), ctypes.byref(g.s), _p64(cw),
                                    _p8(levels))
    return cw, levels, g


def tensor_eval_vector(point, cols, rows, rate, my_id):
    out = fe_array(rows)
    lib().orc_tensor_eval_vector(ctypes.c_uint32(point[0]), ctypes.c_uint32(point[1]), ctypes.c_int(cols),
                                 ctypes.c_int64(rows), ctypes.c_int(rate), ctypes.c_int(my_id), _p64(out))
    return out


def pcs_phase3(B, queries, s, N, rate, my_id):
    B = np.array(np.asarray(B, dtype=np.uint64).reshape(-1, 2), copy=True)
    q = np.ascontiguousarray(queries, dtype=np.uint32).reshape(-1, 2)
    ss = np.ascontiguousarray(s, dtype=np.uint64).reshape(2)
    lib().orc_pcs_phase3(_p64(B), ctypes.c_int64(B.shape[0]), ctypes.c_void_p(q.ctypes.data), ctypes.c_int(q.shape[0]), _p64(ss),
                         ctypes.c_int(N), ctypes.c_int(rate), ctypes.c_int(my_id))
    return B


def encode_concatenated(data, rate0, rate1, degree):
    """encode_concatenated (coPCS.cpp:653-677): (C', C rows)."""
    data = np.ascontiguousarray(data, dtype=np.uint64).reshape(-1, 2)
    n = data.shape[0]
    L = n * rate0
    Cp = fe_array(L)
    C = np.zeros((L // degree, degree * rate1, 2), dtype=np.uint64)
    lib().orc_encode_concatenated(_p64(data), ctypes.c_int64(n), ctypes.c_int(rate0), ctypes.c_int(rate1),
                                  ctypes.c_int(degree), _p64(Cp), _p64(C))
    return Cp, C


def whir_batch_schedule(sizes, rate, whir_k=4):
    """Schedule of Whir_Batch_Open (Whir.cpp:731-752 and the loop of
    :761-833) for polynomials of the given non-increasing sizes: returns
    (kappas, aggr flags, codeword length per array, transcript bytes), or
    None when the reference cannot run the input."""
    k = len(sizes)
    sz = np.ascontiguousarray(sizes, dtype=np.int64)
    kap, agg = np.zeros(64, dtype=np.int32), np.zeros(64, dtype=np.int32)
    cwl, nb = np.zeros(max(k, 1), dtype=np.int64), ctypes.c_int64(0)
    L = lib()
    L.orc_whir_batch_schedule.restype = ctypes.c_int
    n = L.orc_whir_batch_schedule(ctypes.c_int(k), ctypes.c_void_p(sz.ctypes.data), ctypes.c_int(rate),
                                  ctypes.c_int(whir_k), ctypes.c_void_p(kap.ctypes.data),
                                  ctypes.c_void_p(agg.ctypes.data), ctypes.c_void_p(cwl.ctypes.data),
                                  ctypes.byref(nb))
    if n < 0:
        return None
    return [int(x) for x in kap[:n]], [int(x) for x in agg[:n]], [int(x) for x in cwl[:k]], int(nb.value)


def whir_batch_open(arrays, codewords, levels0, betas, K0, rate, whir_k=4, prng_seed=1, prng=None, threads=0):
    """Whir_Batch_Open (Whir.cpp:706-898): returns (transcript bytes,
    final-claim check, prng).  codewords[i] must have the length
    whir_batch_schedule gives for array i (ignored when 0)."""
    arrs = [np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2) for a in arrays]
    bets = [np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 2) for a in betas]
    sizes = [a.shape[0] for a in arrs]
    sch = whir_batch_schedule(sizes, rate, whir_k)
    if sch is None:
        raise ValueError("Whir_Batch_Open cannot run these sizes")
    cws = []
    for i, c in enumerate(codewords):
        cws.append(np.ascontiguousarray(c, dtype=np.uint64).reshape(-1, 2) if c is not None
                   else np.zeros((1, 2), dtype=np.uint64))
    lv = np.ascontiguousarray(levels0, dtype=np.uint8)
    K0 = np.ascontiguousarray(K0, dtype=np.uint64).reshape(2)
    g = prng if prng is not None else Prng(prng_seed)
    out = np.zeros(sch[3], dtype=np.uint8)
    ok = ctypes.c_int(0)
    sz = np.ascontiguousarray(sizes, dtype=np.int64)
    L = lib()
    L.orc_whir_batch_open.restype = ctypes.c_int64
    n = L.orc_whir_batch_open(ctypes.c_int(len(arrs)), _ptr_array(arrs), ctypes.c_void_p(sz.ctypes.data),
                              _ptr_array(cws), _p8(lv), _ptr_array(bets), _p64(K0), ctypes.c_int(rate),
                              ctypes.c_int(whir_k), ctypes.byref(g.s), _p8(out), ctypes.c_int64(out.size),
                              ctypes.byref(ok), ctypes.c_int(threads))
    if n != out.size:
        raise RuntimeError("batch open transcript length %d, expected %d" % (n, out.size))
    return out.tobytes(), bool(ok.value), g

