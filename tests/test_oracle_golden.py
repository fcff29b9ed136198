"""The CPU oracle against golden vectors written by the reference itself.

Pins oracle/gbz_oracle.c: every fixture under tests/golden/ was produced by
the unmodified reference sources (oracle/ref/ref_driver.cpp) through
tests/golden/make_golden.py.  CPU only.
"""
import ctypes
import ctypes.util
import hashlib
import struct

import numpy as np
import pytest

from conftest import golden_bytes, splitmix_base, splitmix_ext

P = (1 << 61) - 1


def fe_from(buf, off, n):
    a = np.frombuffer(buf, dtype=np.uint64, count=2 * n, offset=off).reshape(n, 2)
    return a.copy(), off + 16 * n


def test_field_ops_golden(oracle, golden):
    buf = golden_bytes(golden["field"]["file"])
    (n,) = struct.unpack_from("<I", buf, 0)
    rec = np.frombuffer(buf, dtype=np.uint64, count=14 * n, offset=4).reshape(n, 7, 2)
    a, b = rec[:, 0].copy(), rec[:, 1].copy()
    add, sub, mul, neg, inv = oracle.field_ops(a, b)
    assert np.array_equal(add, rec[:, 2])
    assert np.array_equal(sub, rec[:, 3])
    assert np.array_equal(mul, rec[:, 4])
    assert np.array_equal(neg, rec[:, 5])
    # inv(0) is 0^(p^2-2) = 0 in the reference too
    assert np.array_equal(inv, rec[:, 6])
    roots = np.frombuffer(buf, dtype=np.uint64, count=2 * 62, offset=4 + 16 * 7 * n).reshape(62, 2)
    for lg in range(62):
        assert np.array_equal(oracle.root_of_unity(lg), roots[lg]), lg


def test_blake3_golden(oracle, golden):
    buf = golden_bytes(golden["blake3"]["file"])
    (n,) = struct.unpack_from("<I", buf, 0)
    rec = np.frombuffer(buf, dtype=np.uint8, count=96 * n, offset=4).reshape(n, 96)
    out = oracle.blake3_64(rec[:, :64])
    assert np.array_equal(out, rec[:, 64:])


def test_fiat_shamir_golden(oracle, golden):
    buf = golden_bytes(golden["fs"]["file"])
    cnt = golden["fs"]["count"]
    inp, off = fe_from(buf, 0, cnt)
    # groups of 1, 2, 3, 1, 2, 3 elements
    groups, i, g = [], 0, 1
    while i < cnt:
        groups.append(inp[i:i + g])
        i += g
        g = g % 3 + 1
    outs, off = fe_from(buf, off, len(groups))
    state = np.zeros(2, dtype=np.uint64)
    for k, grp in enumerate(groups):
        assert np.array_equal(oracle.hash_to_field(state, grp), outs[k])
    # get_indexes(8, 2^10, 2^12, -1) (Fiat_Shamir.cpp:37-56)
    for k in range(8):
        state[:] = oracle.hash_F(state, state)
        i0, i1 = struct.unpack_from("<II", buf, off + 8 * k)
        assert (int(state[0]) % (1 << 10), int(state[1]) % (1 << 12)) == (i0, i1)
    off += 64
    final, _ = fe_from(buf, off, 1)
    assert np.array_equal(state, final[0])


@pytest.mark.parametrize("seed", [1, 3396, 42, 123457])
def test_prng_golden(oracle, golden, seed):
    buf = golden_bytes(golden["prng"][str(seed)]["file"])
    cnt = golden["prng"][str(seed)]["count"]
    ref, off = fe_from(buf, 0, cnt)
    g = oracle.Prng(seed)
    for k in range(cnt):
        assert np.array_equal(g.field(), ref[k]), k
    rands = struct.unpack_from("<16i", buf, off)
    assert tuple(g.next() for _ in range(16)) == rands


def test_prng_matches_this_libc():
    """The replica also equals this machine's glibc random() (seeded)."""
    import sys
    sys.path.insert(0, __import__("conftest").ORACLE_DIR)
    import gbz_oracle
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srandom.argtypes = [ctypes.c_uint]
    libc.random.restype = ctypes.c_long
    for seed in (1, 7, 2**31 - 1, 0xDEADBEEF):
        libc.srandom(seed)
        g = gbz_oracle.Prng(seed)
        assert [g.next() for _ in range(500)] == [libc.random() for _ in range(500)]


def test_beta_golden(oracle, golden):
    buf = golden_bytes(golden["beta"]["file"])
    lg = golden["beta"]["logn"]
    r, off = fe_from(buf, 0, lg)
    B, off = fe_from(buf, off, 1 << lg)
    v, off = fe_from(buf, off, 1 << lg)
    e, off = fe_from(buf, off, 1)
    r2, off = fe_from(buf, off, lg)
    bi, off = fe_from(buf, off, 1)
    assert np.array_equal(oracle.precompute_beta(r), B)
    assert np.array_equal(oracle.evaluate_vector(v, r), e[0])
    assert np.array_equal(oracle.beta_identity(r, r2), bi[0])


def test_rs_fold_tensor_golden(oracle, golden):
    g = golden["tensor"]
    buf = golden_bytes(g["file"])
    (cnt,) = struct.unpack_from("<I", buf, 0)
    off = 4
    k = 1 << g["logk"]
    for _ in range(cnt):
        (idx,) = struct.unpack_from("<i", buf, off)
        off += 4
        seg, off = fe_from(buf, off, k)
        r, off = fe_from(buf, off, g["logk"])
        y, off = fe_from(buf, off, 1)
        assert np.array_equal(oracle.rs_fold_tensor(seg, r, 1 << g["logn"], idx), y[0])


def test_update_betas_golden(oracle, golden):
    g = golden["betas"]
    buf = golden_bytes(g["file"])
    nb = 1 << g["logb"]
    b, off = fe_from(buf, 0, nb)
    q = np.frombuffer(buf, dtype=np.int32, count=g["l"], offset=off).copy()
    off += 4 * g["l"]
    ch, off = fe_from(buf, off, g["l"])
    b2, off = fe_from(buf, off, nb)
    r = oracle.Prng(g["prng_seed"]).field()  # update_betas draws one F::_random first
    out, ch2 = oracle.update_betas(b, q, 1 << g["logN"], r)
    assert np.array_equal(ch2, ch)
    assert np.array_equal(out, b2)


def test_fft_golden_files(oracle, golden):
    for e in golden["fft"]:
        if "file" not in e:
            continue
        buf = golden_bytes(e["file"])
        n = 1 << e["logn"]
        a, off = fe_from(buf, 0, n)
        out, _ = fe_from(buf, off, n)
        assert np.array_equal(a, splitmix_ext(e["seed"], n))
        assert np.array_equal(oracle.fft(a, inverse=e["inverse"]), out)


def test_fft_golden_digests(oracle, golden):
    for e in golden["fft"]:
        if "sha256" not in e:
            continue
        n = 1 << e["logn"]
        a = splitmix_ext(e["seed"], n)
        out = oracle.fft(a, inverse=e["inverse"])
        assert hashlib.sha256(a.tobytes() + out.tobytes()).hexdigest() == e["sha256"], e


def _merkle_bytes(a, levels_flat, N):
    parts = [a.tobytes(), struct.pack("<I", (N // 4).bit_length())]
    off, cnt = 0, N // 4
    while cnt >= 1:
        parts.append(struct.pack("<I", cnt))
        parts.append(levels_flat[off:off + cnt].tobytes())
        off += cnt
        cnt //= 2
    return b"".join(parts)


def test_merkle_golden(oracle, golden):
    for e in golden["merkle"]:
        N = 1 << e["logN"]
        a = splitmix_ext(e["seed"], N)
        if N < 4:
            continue  # MT_commit_Blake's N <= 2 branch is not used by the prover
        flat = oracle.merkle_commit(a)
        blob = _merkle_bytes(a, flat, N)
        if "file" in e:
            assert blob == golden_bytes(e["file"])
        else:
            assert hashlib.sha256(blob).hexdigest() == e["sha256"], e


def test_merkle_open_matches_levels(oracle):
    N = 64
    a = splitmix_ext(99, N)
    flat = oracle.merkle_commit(a)
    path = oracle.merkle_open(flat, N, 5)
    assert path.shape == (4, 32)
    assert np.array_equal(path[0], flat[4])          # sibling of leaf 5 is leaf 4
    assert np.array_equal(path[1], flat[16 + 3])     # level 1: sibling of 2 is 3


def test_prove_golden_full(oracle, golden):
    e = golden["prove"][0]
    w = splitmix_base(e["seed"], 1 << e["logn"])
    assert oracle.prove(w, e["logn"], e["rate"], e["prng_seed"]) == golden_bytes(e["file"])


@pytest.mark.parametrize("idx", range(1, 11))
def test_prove_golden_digests(oracle, golden, idx):
    e = golden["prove"][idx]
    if e["logn"] > 18:
        pytest.skip("checked on the GPU against the same digest (CPU oracle too slow here)")
    w = splitmix_base(e["seed"], 1 << e["logn"])
    t = oracle.prove(w, e["logn"], e["rate"], e["prng_seed"])
    assert len(t) == e["bytes"]
    assert hashlib.sha256(t).hexdigest() == e["sha256"]


def test_witness_generator_matches(oracle):
    for seed in (0, 1, 0x5EEE0000):
        assert np.array_equal(oracle.witness(seed, 1000), splitmix_base(seed, 1000))
