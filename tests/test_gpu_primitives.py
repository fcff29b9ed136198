"""GPU parity of the libgbz primitives with the oracle and golden vectors.

Every call goes through the C ABI (include/gbz.h); results must be
bit-identical to the CPU oracle, which is itself pinned to the reference.
"""
import hashlib
import struct

import numpy as np
import pytest

from conftest import splitmix_base, edge_fe, golden_bytes, rand_fe, splitmix_ext

pytestmark = pytest.mark.gpu


def test_field_ops_edge_and_random(ctx, oracle):
    rng = np.random.default_rng(11)
    a, b = edge_fe()
    a = np.concatenate([a, rand_fe(rng, 1 << 16)])
    b = np.concatenate([b, rand_fe(rng, 1 << 16)])
    s, d, p = ctx.field_ops(a, b)
    os_, od, op, _, _ = oracle.field_ops(a, b)
    assert np.array_equal(s, os_)
    assert np.array_equal(d, od)
    assert np.array_equal(p, op)


def test_field_ops_golden(ctx, golden):
    buf = golden_bytes(golden["field"]["file"])
    (n,) = struct.unpack_from("<I", buf, 0)
    rec = np.frombuffer(buf, dtype=np.uint64, count=14 * n, offset=4).reshape(n, 7, 2)
    s, d, p = ctx.field_ops(rec[:, 0].copy(), rec[:, 1].copy())
    assert np.array_equal(s, rec[:, 2])
    assert np.array_equal(d, rec[:, 3])
    assert np.array_equal(p, rec[:, 4])


def test_blake3_golden(ctx, golden):
    buf = golden_bytes(golden["blake3"]["file"])
    (n,) = struct.unpack_from("<I", buf, 0)
    rec = np.frombuffer(buf, dtype=np.uint8, count=96 * n, offset=4).reshape(n, 96)
    assert np.array_equal(ctx.blake3_hash(rec[:, :64].copy()), rec[:, 64:])


def test_blake3_random_vs_oracle(ctx, oracle):
    rng = np.random.default_rng(12)
    blocks = rng.integers(0, 256, size=(5000, 64), dtype=np.uint8)
    assert np.array_equal(ctx.blake3_hash(blocks), oracle.blake3_64(blocks))


@pytest.mark.parametrize("logn", list(range(0, 15)) + [16, 18, 20])
@pytest.mark.parametrize("inverse", [False, True])
def test_fft_vs_oracle(ctx, oracle, logn, inverse):
    a = splitmix_ext(1000 + logn, 1 << logn)
    got = ctx.fft(a.copy(), logn, inverse)
    assert np.array_equal(got, oracle.fft(a, inverse=inverse))


def test_fft_golden(ctx, golden):
    for e in golden["fft"]:
        n = 1 << e["logn"]
        a = splitmix_ext(e["seed"], n)
        out = ctx.fft(a.copy(), e["logn"], e["inverse"])
        if "file" in e:
            assert out.tobytes() == golden_bytes(e["file"])[16 * n:]
        else:
            assert hashlib.sha256(a.tobytes() + out.tobytes()).hexdigest() == e["sha256"], e


@pytest.mark.parametrize("logn", [21, 22, 23, 24, 25])
def test_fft_roundtrip_large(ctx, logn):
    """Size-independent property at full sizes: inverse(forward(x)) == x."""
    a = splitmix_ext(77 + logn, 1 << logn)
    b = ctx.fft(a.copy(), logn, False)
    assert not np.array_equal(a, b)
    c = ctx.fft(b, logn, True)
    assert np.array_equal(a, c)


def test_fft_linearity_large(ctx, oracle):
    logn = 23
    rng = np.random.default_rng(3)
    x, y = rand_fe(rng, 1 << logn), rand_fe(rng, 1 << logn)
    fx, fy = ctx.fft(x.copy(), logn, False), ctx.fft(y.copy(), logn, False)
    s, _, _ = ctx.field_ops(x, y)
    fs = ctx.fft(s, logn, False)
    fxy, _, _ = ctx.field_ops(fx, fy)
    assert np.array_equal(fs, fxy)


@pytest.mark.parametrize("logm,rate", [(2, 2), (5, 4), (10, 2), (12, 4), (14, 8), (17, 2)])
def test_rs_encode_vs_oracle(ctx, oracle, logm, rate):
    a = splitmix_ext(5 + logm, 1 << logm)
    padded = np.zeros(((1 << logm) * rate, 2), dtype=np.uint64)
    padded[: 1 << logm] = a
    assert np.array_equal(ctx.rs_encode(a, rate), oracle.fft(padded))


@pytest.mark.parametrize("logm,rate", [(1, 2), (2, 2), (5, 4), (10, 2), (12, 4), (13, 2), (14, 8), (17, 2), (20, 2)])
def test_rs_encode_base_field_vs_oracle(ctx, oracle, logm, rate):
    """Base-field coefficients take the packed real-input transform."""
    a = splitmix_base(15 + logm, 1 << logm)
    padded = np.zeros(((1 << logm) * rate, 2), dtype=np.uint64)
    padded[: 1 << logm] = a
    assert np.array_equal(ctx.rs_encode(a, rate), oracle.fft(padded))


def test_whir_commit_base_field(ctx, oracle):
    a = splitmix_base(18, 1 << 12)
    cw, flat = ctx.Whir_Commit_initial(a, 2)
    padded = np.zeros((1 << 13, 2), dtype=np.uint64)
    padded[: 1 << 12] = a
    ocw = oracle.fft(padded)
    assert np.array_equal(cw, ocw)
    assert np.array_equal(flat, oracle.merkle_commit(ocw))


@pytest.mark.parametrize("logN", [2, 3, 4, 5, 8, 11, 12, 13, 14, 15, 16])
def test_merkle_vs_oracle(ctx, oracle, logN):
    a = splitmix_ext(300 + logN, 1 << logN)
    assert np.array_equal(ctx.merkle_commit_flat(a), oracle.merkle_commit(a))


def test_merkle_golden(ctx, golden):
    for e in golden["merkle"]:
        N = 1 << e["logN"]
        if N < 4:
            continue
        a = splitmix_ext(e["seed"], N)
        flat = ctx.merkle_commit_flat(a)
        parts = [a.tobytes(), struct.pack("<I", (N // 4).bit_length())]
        off, cnt = 0, N // 4
        while cnt >= 1:
            parts += [struct.pack("<I", cnt), flat[off:off + cnt].tobytes()]
            off += cnt
            cnt //= 2
        blob = b"".join(parts)
        if "file" in e:
            assert blob == golden_bytes(e["file"])
        else:
            assert hashlib.sha256(blob).hexdigest() == e["sha256"], e


def test_merkle_large_levels_consistent(ctx, oracle):
    """2^22 elements: spot-check nodes of every level against the oracle's
    hash of the left child (the whole tree is too slow for the CPU)."""
    logN = 22
    N = 1 << logN
    a = splitmix_ext(4242, N)
    flat = ctx.merkle_commit_flat(a)
    rng = np.random.default_rng(9)
    leaves = rng.integers(0, N // 4, size=64)
    blocks = a.reshape(N // 4, 64 // 16 * 2)[leaves].view(np.uint8).reshape(-1, 64)
    assert np.array_equal(flat[leaves], oracle.blake3_64(blocks))
    off, cnt = 0, N // 4
    while cnt > 1:
        nxt = off + cnt
        idx = rng.integers(0, cnt // 2, size=32)
        child = flat[off + 2 * idx]
        blk = np.concatenate([child, child], axis=1)
        assert np.array_equal(flat[nxt + idx], oracle.blake3_64(blk))
        off, cnt = nxt, cnt // 2


def test_whir_commit_and_open(ctx, oracle, gbz):
    a = splitmix_ext(8, 1 << 12)
    cw, flat = ctx.Whir_Commit_initial(a, 4)
    padded = np.zeros((1 << 14, 2), dtype=np.uint64)
    padded[: 1 << 12] = a
    ocw = oracle.fft(padded)
    assert np.array_equal(cw, ocw)
    assert np.array_equal(flat, oracle.merkle_commit(ocw))
    for pos in (0, 1, 77, (1 << 12) - 1):
        assert np.array_equal(gbz.open_tree_blake(flat, 1 << 14, pos), oracle.merkle_open(flat, 1 << 14, pos))


@pytest.mark.parametrize("nr", [0, 1, 3, 4, 5, 10, 17])
def test_precompute_beta_vs_oracle(ctx, oracle, nr):
    r = splitmix_ext(50 + nr, max(nr, 1))[:nr]
    assert np.array_equal(ctx.precompute_beta(r), oracle.precompute_beta(r))


def test_precompute_beta_golden(ctx, golden):
    buf = golden_bytes(golden["beta"]["file"])
    lg = golden["beta"]["logn"]
    r = np.frombuffer(buf, dtype=np.uint64, count=2 * lg).reshape(lg, 2).copy()
    B = np.frombuffer(buf, dtype=np.uint64, count=2 << lg, offset=16 * lg).reshape(-1, 2)
    assert np.array_equal(ctx.precompute_beta(r), B)


@pytest.mark.parametrize("logm", [1, 2, 3, 8, 12, 16, 20])
def test_sumcheck_round_and_fold(ctx, oracle, logm):
    rng = np.random.default_rng(logm)
    v1, v2 = rand_fe(rng, 1 << logm), rand_fe(rng, 1 << logm)
    assert np.array_equal(ctx.whir_sumcheck_step1(v1, v2), oracle.sumcheck_quadratic(v1, v2))
    r = rand_fe(rng, 1)[0]
    assert np.array_equal(ctx.sumcheck_fold(v1, r), oracle.sumcheck_fold(v1, r))


def test_update_betas_golden(ctx, oracle, golden):
    g = golden["betas"]
    buf = golden_bytes(g["file"])
    nb = 1 << g["logb"]
    b = np.frombuffer(buf, dtype=np.uint64, count=2 * nb).reshape(nb, 2).copy()
    off = 16 * nb
    q = np.frombuffer(buf, dtype=np.int32, count=g["l"], offset=off).copy()
    off += 4 * g["l"]
    ch = np.frombuffer(buf, dtype=np.uint64, count=2 * g["l"], offset=off).reshape(-1, 2)
    off += 16 * g["l"]
    b2 = np.frombuffer(buf, dtype=np.uint64, count=2 * nb, offset=off).reshape(nb, 2)
    r = oracle.Prng(g["prng_seed"]).field()
    out, ch2 = ctx.update_betas(b, q, 1 << g["logN"], r)
    assert np.array_equal(ch2, ch)
    assert np.array_equal(out, b2)


@pytest.mark.parametrize("logb,logN,l,dups", [(3, 6, 5, 0), (10, 13, 100, 0), (14, 16, 200, 0), (16, 19, 33, 0),
                                               (1, 4, 7, 0), (15, 17, 150, 1), (20, 22, 200, 1), (18, 20, 16, 0)])
def test_update_betas_vs_oracle(ctx, oracle, logb, logN, l, dups):
    """Direct sums and the sparse-transform path (chosen by size); dups puts
    several queries on the same position and in the same column."""
    rng = np.random.default_rng(logb * 7 + l)
    b = rand_fe(rng, 1 << logb)
    q = rng.integers(0, 1 << logN, size=l).astype(np.int32)
    if dups:
        q[1::3] = q[0]
        q[2::5] = (q[0] + (1 << (logN // 2 + 1))) % (1 << logN)
    r = rand_fe(rng, 1)[0]
    out, ch = ctx.update_betas(b, q, 1 << logN, r)
    ob, och = oracle.update_betas(b, q, 1 << logN, r)
    assert np.array_equal(ch, och)
    assert np.array_equal(out, ob)


def test_invalid_arguments_return_einval(ctx, gbz):
    with pytest.raises(gbz.GbzError) as e:
        ctx.rs_encode(np.zeros((3, 2), dtype=np.uint64), 2)
    assert e.value.status == gbz.EINVAL
    with pytest.raises(gbz.GbzError) as e:
        ctx.merkle_commit_flat(np.zeros((2, 2), dtype=np.uint64))
    assert e.value.status == gbz.EINVAL
    small = np.zeros((4, 2), dtype=np.uint64)
    assert gbz.lib.gbz_fft(ctx.h, small.ctypes.data, 29, 0, gbz.MEM_HOST) == gbz.EINVAL
    assert gbz.lib.gbz_fft(ctx.h, None, 2, 0, gbz.MEM_HOST) == gbz.EINVAL
    assert gbz.lib.gbz_fft(ctx.h, small.ctypes.data, 2, 0, 7) == gbz.EINVAL
