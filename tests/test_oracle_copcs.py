"""The CPU oracle's coPCS-side functions against the reference's own outputs.

Fixtures come from oracle/ref/ref_full_driver.cpp, which links every
reference translation unit except main.cpp (tests/golden/make_golden.py).
CPU only.
"""
import struct

import numpy as np
import pytest

from conftest import golden_bytes, splitmix_ext


class Reader:
    def __init__(self, buf):
        self.buf, self.off = buf, 0

    def fe(self, n):
        a = np.frombuffer(self.buf, dtype=np.uint64, count=2 * n, offset=self.off).reshape(n, 2).copy()
        self.off += 16 * n
        return a

    def u32(self):
        (v,) = struct.unpack_from("<I", self.buf, self.off)
        self.off += 4
        return v

    def raw(self, n):
        b = self.buf[self.off:self.off + n]
        self.off += n
        return b

    def done(self):
        assert self.off == len(self.buf)


def case(golden, name):
    e = golden["copcs"][name]
    return Reader(golden_bytes(e["file"])), e["args"]


@pytest.mark.parametrize("name", ["multifold5_10_2", "multifold5_12_3", "multifold5_9_1"])
def test_rs_multifold5(oracle, golden, name):
    r, (_, logn, logd, seed) = case(golden, name)
    cw, a, out = r.fe(1 << logn), r.fe(1 << logd), r.fe(1 << (logn - logd))
    r.done()
    assert np.array_equal(cw, splitmix_ext(seed, 1 << logn))
    assert np.array_equal(oracle.rs_multifold5(cw, a), out)


@pytest.mark.parametrize("name", ["lagrange_4", "lagrange_7"])
def test_lagrange(oracle, golden, name):
    r, (_, logd, _) = case(golden, name)
    rr, out = r.fe(1), r.fe(1 << logd)
    r.done()
    assert np.array_equal(oracle.lagrange_coeff(rr[0], logd), out)


@pytest.mark.parametrize("name", ["encode_3_8", "encode_5_6"])
def test_encode(oracle, golden, name):
    r, (_, rows, logrow, rate, log_ro, _) = case(golden, name)
    n = 1 << logrow
    inp = np.stack([r.fe(n) for _ in range(rows)])
    out = np.stack([r.fe(n * rate) for _ in range(rows)])
    r.done()
    assert np.array_equal(oracle.encode_rows(inp, rate, log_ro), out)


@pytest.mark.parametrize("name", ["colmerkle_5_8", "colmerkle_2_6", "colmerkle_32_5"])
def test_column_merkle(oracle, golden, name):
    r, (_, rows, logL, N, _) = case(golden, name)
    L = 1 << logL
    inp = np.stack([r.fe(L) for _ in range(rows)])
    nlv = r.u32()
    levels = []
    for _ in range(nlv):
        cnt = r.u32()
        levels.append(np.frombuffer(r.raw(32 * cnt), dtype=np.uint8).reshape(cnt, 32))
    root = np.frombuffer(r.raw(32), dtype=np.uint8)
    r.done()
    got_levels, got_root = oracle.column_merkle(inp, N)
    assert np.array_equal(got_levels, np.concatenate(levels))
    assert np.array_equal(got_root, root)


@pytest.mark.parametrize("name", ["shares_8_16", "shares_9_16p", "shares_7_8p"])
def test_secret_shares(oracle, golden, name):
    r, (_, logM, N, _, privacy, prng_seed) = case(golden, name)
    M = 1 << logM
    v = r.fe(M)
    shares = np.stack([r.fe(M // (N // 4)) for _ in range(N)])
    r.done()
    assert np.array_equal(oracle.secret_shares(v, N, bool(privacy), prng_seed), shares)


@pytest.mark.parametrize("name", ["aggr_16_24", "aggr_8_10", "aggr_32_6"])
def test_party_aggregate(oracle, golden, name):
    r, (_, N, length, _) = case(golden, name)
    msgs = np.stack([r.fe(length) for _ in range(N)])
    b = r.fe(N // 4)
    out = r.fe(length)
    r.done()
    assert np.array_equal(oracle.party_aggregate(msgs, b), out)


@pytest.mark.parametrize("name", ["cophase1_10_3", "cophase1_9_2"])
def test_cophase1(oracle, golden, name):
    r, (_, logn, logd, _) = case(golden, name)
    n, d = 1 << logn, 1 << logd
    p1, p2, p3, b1 = r.fe(n), r.fe(n), r.fe(n), r.fe(n)
    H, H4 = r.fe(2 * d), r.fe(4 * d)
    r.done()
    gH, gH4 = oracle.cophase1(p1, p2, p3, b1, logd)
    assert np.array_equal(gH, H)
    assert np.array_equal(gH4, H4)


@pytest.mark.parametrize("name", ["cophase2_10_3", "cophase2_8_4"])
def test_cophase2(oracle, golden, name):
    r, (_, logn, logd, _) = case(golden, name)
    n, d = 1 << logn, 1 << logd
    p1, p2, p3, b1, L = r.fe(n), r.fe(n), r.fe(n), r.fe(n), r.fe(d)
    q1, q2 = r.fe(n // d), r.fe(n // d)
    c1, c2, c3, c4 = r.fe(n // d), r.fe(n // d), r.fe(n // d), r.fe(n // d)
    r.done()
    assert np.array_equal(oracle.cophase2(p1, L), q1)
    assert np.array_equal(oracle.cophase2(p2, L), q2)
    for v, ref in ((p1, c1), (p2, c2), (p3, c3), (b1, c4)):
        assert np.array_equal(oracle.cophase2(v, L), ref)
