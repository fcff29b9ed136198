"""GPU parity of the collaborative-PCS side with the oracle and the golden
vectors written by the reference (RS folding, Lagrange weights, coPCS
encoding, per-column Merkle roots, packed Shamir shares, the leader's
aggregation and the block-univariate sumcheck rounds).

Every call goes through the C ABI; results must be bit-identical.
"""
import numpy as np
import pytest

from conftest import splitmix_base, rand_fe, splitmix_ext
from test_oracle_copcs import case

pytestmark = pytest.mark.gpu


# ------------------------------------------------------------ RS_multifold5
@pytest.mark.parametrize("name", ["multifold5_10_2", "multifold5_12_3", "multifold5_9_1"])
def test_rs_multifold5_golden(ctx, golden, name):
    r, (_, logn, logd, seed) = case(golden, name)
    cw, a, out = r.fe(1 << logn), r.fe(1 << logd), r.fe(1 << (logn - logd))
    assert np.array_equal(cw, splitmix_ext(seed, 1 << logn))
    assert np.array_equal(ctx.RS_multifold5(cw, a), out)


@pytest.mark.parametrize("logn,logd", [(5, 1), (6, 4), (11, 4), (13, 2), (16, 3), (20, 4), (22, 1)])
def test_rs_multifold5_vs_oracle(ctx, oracle, logn, logd):
    rng = np.random.default_rng(100 + logn * 8 + logd)
    cw, a = rand_fe(rng, 1 << logn), rand_fe(rng, 1 << logd)
    assert np.array_equal(ctx.RS_multifold5(cw, a), oracle.rs_multifold5(cw, a))


def test_rs_multifold5_low_degree(ctx, oracle):
    """A codeword of a low-degree polynomial folds to a codeword again: the
    fold of an RS codeword with all-ones weights is an RS codeword of the
    folded polynomial (size-independent property at 2^24)."""
    logn, logd = 24, 4
    n = 1 << logn
    rng = np.random.default_rng(7)
    coeffs = rand_fe(rng, 1 << 10)
    cw = ctx.rs_encode(coeffs, n >> 10)
    a = rand_fe(rng, 1 << logd)
    folded = ctx.RS_multifold5(cw, a)
    # the folded word is the evaluation of a polynomial of degree < 2^10 / 16
    back = ctx.fft(folded.copy(), logn - logd, True)
    assert not np.any(back[(1 << 10) >> logd:])
    # and it agrees with the oracle on a sample of positions
    assert np.array_equal(folded[:4096], oracle.rs_multifold5(cw, a)[:4096])


def test_rs_multifold5_invalid(ctx, gbz):
    with pytest.raises(gbz.GbzError):
        ctx.RS_multifold5(np.zeros((1 << 8, 2), np.uint64), np.zeros((32, 2), np.uint64))
    with pytest.raises(gbz.GbzError):
        ctx.RS_multifold5(np.zeros((12, 2), np.uint64), np.zeros((2, 2), np.uint64))


# ---------------------------------------------------------------- Lagrange
@pytest.mark.parametrize("name", ["lagrange_4", "lagrange_7"])
def test_lagrange_golden(ctx, golden, name):
    r, (_, logd, _) = case(golden, name)
    rr, out = r.fe(1), r.fe(1 << logd)
    assert np.array_equal(ctx.compute_lagrange_coeff(rr[0], logd), out)


@pytest.mark.parametrize("logd", [0, 1, 3, 9, 13, 16])
def test_lagrange_vs_oracle(ctx, oracle, logd):
    rng = np.random.default_rng(200 + logd)
    r = rand_fe(rng, 1)[0]
    assert np.array_equal(ctx.compute_lagrange_coeff(r, logd), oracle.lagrange_coeff(r, logd))


# ------------------------------------------------------------------ Encode
@pytest.mark.parametrize("name", ["encode_3_8", "encode_5_6"])
def test_encode_golden(ctx, golden, name):
    r, (_, rows, logrow, rate, log_ro, _) = case(golden, name)
    n = 1 << logrow
    inp = np.stack([r.fe(n) for _ in range(rows)])
    out = np.stack([r.fe(n * rate) for _ in range(rows)])
    assert np.array_equal(ctx.Encode(inp, rate, log_ro), out)


@pytest.mark.parametrize("rows,logrow,rate,log_ro", [(1, 0, 2, 0), (2, 1, 4, 3), (3, 10, 2, 1), (2, 12, 8, 5),
                                                     (1, 14, 2, 2), (1, 16, 4, 4),
                                                     # rate 2, offset 0: half-length transform + the row itself
                                                     (1, 1, 2, 0), (3, 5, 2, 0), (2, 13, 2, 0), (2, 14, 2, 0),
                                                     (16, 12, 2, 0), (1, 18, 2, 0)])
def test_encode_vs_oracle(ctx, oracle, rows, logrow, rate, log_ro):
    rng = np.random.default_rng(300 + logrow)
    inp = np.stack([rand_fe(rng, 1 << logrow) for _ in range(rows)])
    assert np.array_equal(ctx.Encode(inp, rate, log_ro), oracle.encode_rows(inp, rate, log_ro))


@pytest.mark.parametrize("rows,logrow,rate,log_ro", [(1, 2, 2, 0), (3, 5, 2, 0), (2, 10, 4, 1), (16, 12, 2, 0),
                                                     (2, 13, 2, 0), (2, 14, 2, 0), (4, 14, 8, 2), (1, 18, 2, 0)])
def test_encode_base_field_rows_vs_oracle(ctx, oracle, rows, logrow, rate, log_ro):
    """Base-field rows, as the party shares of the configurations are."""
    inp = np.stack([splitmix_base(700 + 31 * k + logrow, 1 << logrow) for k in range(rows)])
    assert np.array_equal(ctx.Encode(inp, rate, log_ro), oracle.encode_rows(inp, rate, log_ro))


def test_encode_mixed_rows_vs_oracle(ctx, oracle):
    """Base-field rows, then the same rows with one imaginary word, then the
    base-field rows again: every call matches the oracle."""
    logrow = 13
    base = np.stack([splitmix_base(900 + k, 1 << logrow) for k in range(3)])
    mixed = base.copy()
    mixed[2, 4095, 1] = 7
    for inp in (base, mixed, base):
        assert np.array_equal(ctx.Encode(inp, 2, 0), oracle.encode_rows(inp, 2, 0))


def test_encode_large_is_low_degree(ctx):
    """A 2^22-entry codeword interpolates to a polynomial whose
    coefficients vanish above the row length (coset scaling keeps degree)."""
    logrow, rate = 21, 2
    rng = np.random.default_rng(301)
    inp = rand_fe(rng, 1 << logrow)[None]
    cw = ctx.Encode(inp, rate, 3)[0]
    back = ctx.fft(cw.copy(), logrow + 1, True)
    assert not np.any(back[1 << logrow:])
    assert np.any(back[: 1 << logrow])


# ----------------------------------------------------------- distributed_MT
@pytest.mark.parametrize("name", ["colmerkle_5_8", "colmerkle_2_6", "colmerkle_32_5"])
def test_column_merkle_golden(ctx, golden, name):
    r, (_, rows, logL, N, _) = case(golden, name)
    L = 1 << logL
    inp = np.stack([r.fe(L) for _ in range(rows)])
    nlv = r.u32()
    levels = []
    for _ in range(nlv):
        cnt = r.u32()
        levels.append(np.frombuffer(r.raw(32 * cnt), dtype=np.uint8).reshape(cnt, 32))
    root = np.frombuffer(r.raw(32), dtype=np.uint8)
    got_levels, got_root = ctx.distributed_MT(inp, N)
    assert np.array_equal(got_levels, np.concatenate(levels))
    assert np.array_equal(got_root, root)


@pytest.mark.parametrize("rows,logL,N", [(1, 0, 1), (3, 1, 2), (4, 9, 64), (7, 12, 4), (32, 15, 32)])
def test_column_merkle_vs_oracle(ctx, oracle, rows, logL, N):
    rng = np.random.default_rng(400 + logL)
    inp = np.stack([rand_fe(rng, 1 << logL) for _ in range(rows)])
    gl, gr = ctx.distributed_MT(inp, N)
    ol, orr = oracle.column_merkle(inp, N)
    assert np.array_equal(gl, ol)
    assert np.array_equal(gr, orr)


# ------------------------------------------------------- Shamir shares
@pytest.mark.parametrize("name", ["shares_8_16", "shares_9_16p", "shares_7_8p"])
def test_secret_shares_golden(ctx, golden, name):
    r, (_, logM, N, _, privacy, prng_seed) = case(golden, name)
    M = 1 << logM
    v = r.fe(M)
    shares = np.stack([r.fe(M // (N // 4)) for _ in range(N)])
    assert np.array_equal(ctx.compute_secret_shares(v, N, bool(privacy), prng_seed), shares)


@pytest.mark.parametrize("logM,N,privacy", [(2, 4, False), (10, 64, True), (16, 32, False), (18, 8, True)])
def test_secret_shares_vs_oracle(ctx, oracle, logM, N, privacy):
    rng = np.random.default_rng(500 + logM)
    v = rand_fe(rng, 1 << logM)
    assert np.array_equal(ctx.compute_secret_shares(v, N, privacy, 3),
                          oracle.secret_shares(v, N, privacy, 3))


def test_shares_then_aggregate_recovers_secrets(ctx):
    """Packing then the leader's aggregation with unit weights recovers the
    secrets' weighted sums: aggregate(shares of v, b) = sum_j b_j v_j per
    group (privacy on: the random fill must not leak into the result)."""
    N, groups = 16, 1 << 12
    k = N // 4
    rng = np.random.default_rng(501)
    v = rand_fe(rng, groups * k)
    sh = ctx.compute_secret_shares(v, N, True, 11)  # (N, groups, 2)
    b = rand_fe(rng, k)
    agg = ctx.sumcheck_aggr(sh, b)
    # expected: sum_j b_j v[i k + j]
    P = (1 << 61) - 1
    vv = v.reshape(groups, k, 2)
    br, bi = [int(x) for x in b[:, 0]], [int(x) for x in b[:, 1]]
    for i in (0, 1, groups - 1):
        re = im = 0
        for j in range(k):
            xr, xi = int(vv[i, j, 0]), int(vv[i, j, 1])
            re += br[j] * xr - bi[j] * xi
            im += br[j] * xi + bi[j] * xr
        assert (int(agg[i, 0]), int(agg[i, 1])) == (re % P, im % P)


# ------------------------------------------------------------ aggregation
@pytest.mark.parametrize("name", ["aggr_16_24", "aggr_8_10", "aggr_32_6"])
def test_party_aggregate_golden(ctx, golden, name):
    r, (_, N, length, _) = case(golden, name)
    msgs = np.stack([r.fe(length) for _ in range(N)])
    b = r.fe(N // 4)
    out = r.fe(length)
    assert np.array_equal(ctx.sumcheck_aggr(msgs, b), out)


@pytest.mark.parametrize("N,length", [(4, 1), (64, 1000), (256, 64), (1024, 3)])
def test_party_aggregate_vs_oracle(ctx, oracle, N, length):
    rng = np.random.default_rng(600 + N)
    msgs = np.stack([rand_fe(rng, length) for _ in range(N)])
    b = rand_fe(rng, N // 4)
    assert np.array_equal(ctx.sumcheck_aggr(msgs, b), oracle.party_aggregate(msgs, b))


# ------------------------------------------------------- coSumcheck rounds
@pytest.mark.parametrize("name", ["cophase1_10_3", "cophase1_9_2"])
def test_cophase1_golden(ctx, golden, name):
    r, (_, logn, logd, _) = case(golden, name)
    n = 1 << logn
    p1, p2, p3, b1 = r.fe(n), r.fe(n), r.fe(n), r.fe(n)
    H, H4 = r.fe(2 << logd), r.fe(4 << logd)
    assert np.array_equal(ctx.coSumcheck_phase1(p1, p2, logd), H)
    assert np.array_equal(ctx.coSumcheck_phase1(p1, p2, logd, p3, b1), H4)


@pytest.mark.parametrize("logn,logd", [(0, 0), (4, 2), (12, 6), (14, 7), (15, 11), (16, 5), (18, 3), (17, 1)])
def test_cophase1_vs_oracle(ctx, oracle, logn, logd):
    rng = np.random.default_rng(700 + logn)
    n = 1 << logn
    p1, p2, p3, b1 = (rand_fe(rng, n) for _ in range(4))
    # zero blocks of p1: skipped by the cubic form, harmless to the quadratic
    d = 1 << logd
    for blk in range(0, n // d, 3):
        p1[blk * d:(blk + 1) * d] = 0
    H, H4 = oracle.cophase1(p1, p2, p3, b1, logd)
    assert np.array_equal(ctx.coSumcheck_phase1(p1, p2, logd), H)
    assert np.array_equal(ctx.coSumcheck_phase1(p1, p2, logd, p3, b1), H4)


def test_cophase1_device_inputs(ctx, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(710)
    logn, logd = 13, 4
    vs = [rand_fe(rng, 1 << logn) for _ in range(4)]
    dv = [torch.from_numpy(v.view(np.int64)).cuda() for v in vs]
    H, H4 = oracle.cophase1(*vs, logd)
    assert np.array_equal(ctx.coSumcheck_phase1(dv[0], dv[1], logd), H)
    assert np.array_equal(ctx.coSumcheck_phase1(dv[0], dv[1], logd, dv[2], dv[3]), H4)


@pytest.mark.parametrize("name", ["cophase2_10_3", "cophase2_8_4"])
def test_cophase2_golden(ctx, golden, name):
    r, (_, logn, logd, _) = case(golden, name)
    n, d = 1 << logn, 1 << logd
    p1, p2, p3, b1, L = r.fe(n), r.fe(n), r.fe(n), r.fe(n), r.fe(d)
    q1, q2 = r.fe(n // d), r.fe(n // d)
    c = [r.fe(n // d) for _ in range(4)]
    assert np.array_equal(ctx.coSumcheck_phase2(p1, L), q1)
    assert np.array_equal(ctx.coSumcheck_phase2(p2, L), q2)
    for v, ref in zip((p1, p2, p3, b1), c):
        assert np.array_equal(ctx.coSumcheck_phase2(v, L), ref)


@pytest.mark.parametrize("logn,logd", [(0, 0), (5, 5), (16, 10), (22, 3)])
def test_cophase2_vs_oracle(ctx, oracle, logn, logd):
    rng = np.random.default_rng(800 + logn)
    v, L = rand_fe(rng, 1 << logn), rand_fe(rng, 1 << logd)
    assert np.array_equal(ctx.coSumcheck_phase2(v, L), oracle.cophase2(v, L))


def test_cosumcheck_round_consistency(ctx):
    """One block-univariate round: with L = Lagrange weights at r, the folded
    vectors' blockwise products sum to H(r) interpolated from phase 1."""
    rng = np.random.default_rng(900)
    logn, logd = 12, 3
    n, d = 1 << logn, 1 << logd
    p1, p2 = rand_fe(rng, n), rand_fe(rng, n)
    H = ctx.coSumcheck_phase1(p1, p2, logd)  # evaluations of sum_blocks ext(p1) ext(p2) on 2d points
    r = rand_fe(rng, 1)[0]
    # evaluate H's interpolant at r: coefficients by inverse transform, then Horner
    coef = ctx.fft(H.copy(), logd + 1, True)
    P = (1 << 61) - 1

    def mul(a, b):
        return ((a[0] * b[0] - a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)

    acc = (0, 0)
    rr = (int(r[0]), int(r[1]))
    for c in coef[::-1]:
        acc = mul(acc, rr)
        acc = ((acc[0] + int(c[0])) % P, (acc[1] + int(c[1])) % P)
    L = ctx.compute_lagrange_coeff(r, logd)
    f1, f2 = ctx.coSumcheck_phase2(p1, L), ctx.coSumcheck_phase2(p2, L)
    s = (0, 0)
    for x, y in zip(f1, f2):
        t = mul((int(x[0]), int(x[1])), (int(y[0]), int(y[1])))
        s = ((s[0] + t[0]) % P, (s[1] + t[1]) % P)
    assert s == acc


@pytest.mark.parametrize("name", ["encconc_8_2_2_4", "encconc_10_4_2_16", "encconc_6_2_4_8"])
def test_encode_concatenated_golden(ctx, golden, name):
    e = golden["sumcheck"][name]
    from conftest import golden_bytes
    from test_oracle_copcs import Reader
    r, (_, logn, rate0, rate1, degree, seed) = Reader(golden_bytes(e["file"])), e["args"]
    n = 1 << logn
    L = n * rate0
    Cp = r.fe(L)
    C = np.stack([r.fe(degree * rate1) for _ in range(L // degree)])
    gCp, gC = ctx.encode_concatenated(splitmix_ext(seed, n), rate0, rate1, degree)
    assert np.array_equal(gCp, Cp)
    assert np.array_equal(gC, C)


@pytest.mark.parametrize("logn,rate0,rate1,degree", [(14, 2, 2, 4), (16, 4, 4, 64), (18, 2, 8, 1024), (12, 8, 2, 4096)])
def test_encode_concatenated_vs_oracle(ctx, oracle, logn, rate0, rate1, degree):
    rng = np.random.default_rng(logn * 7 + degree)
    data = rand_fe(rng, 1 << logn)
    gCp, gC = ctx.encode_concatenated(data, rate0, rate1, degree)
    oCp, oC = oracle.encode_concatenated(data, rate0, rate1, degree)
    assert np.array_equal(gCp, oCp)
    assert np.array_equal(gC, oC)
