"""Shared test fixtures.

-m "not gpu": the oracle against the reference's golden vectors, the host
side of libgbz (exports, protocol helpers, layout), no GPU work.
-m gpu: parity of the CUDA path with the oracle and the golden vectors,
through the C ABI.
"""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "shorter-and-faster-post-quantum-secure-scalable-collaborative-snarks_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")

for p in (PKG, ORACLE_DIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libgbz kernels)")


@pytest.fixture(scope="session")
def oracle():
    import gbz_oracle

    gbz_oracle.build()
    return gbz_oracle


@pytest.fixture(scope="session")
def gbz():
    import build_lib

    build_lib.build()
    import gbz as mod

    return mod


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def golden_bytes(name):
    with open(os.path.join(GOLDEN, name), "rb") as f:
        return f.read()


@pytest.fixture(scope="session")
def ctx(gbz):
    c = gbz.Context(0)
    yield c
    c.close()


class SplitMix:
    """The input generator of oracle/ref/ref_driver.cpp."""

    P = (1 << 61) - 1

    def __init__(self, seed):
        self.s = seed & (2**64 - 1)

    def next(self):
        M = 2**64 - 1
        self.s = (self.s + 0x9E3779B97F4A7C15) & M
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    def base(self):
        while True:
            v = self.next() >> 3
            if v != self.P:
                return v

    def ext_array(self, n):
        out = np.zeros((n, 2), dtype=np.uint64)
        for i in range(n):
            out[i, 0] = self.base()
            out[i, 1] = self.base()
        return out


def rand_fe(rng, n, base=False):
    """Canonical random field elements from a numpy Generator."""
    a = rng.integers(0, (1 << 61) - 1, size=(n, 2), dtype=np.uint64)
    if base:
        a[:, 1] = 0
    return a


def edge_fe():
    """Edge values: 0, 1, p-1, 2, 2^60, 2^32-1, generator parts."""
    P = (1 << 61) - 1
    vals = [0, 1, P - 1, 2, 1 << 60, (1 << 32) - 1, 2147483648, 1033321771269002680, P - 2]
    a, b = [], []
    for x in vals:
        for y in vals:
            a.append((x, y))
            b.append((y, x))
    return np.array(a, dtype=np.uint64), np.array(b, dtype=np.uint64)


def splitmix_words(seed, count):
    """count consecutive SplitMix64 outputs (vectorised)."""
    M = np.uint64
    with np.errstate(over="ignore"):
        s = M(seed) + (np.arange(1, count + 1, dtype=np.uint64) * M(0x9E3779B97F4A7C15))
        z = s.copy()
        z = (z ^ (z >> M(30))) * M(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> M(27))) * M(0x94D049BB133111EB)
        z = z ^ (z >> M(31))
    return z


def splitmix_ext(seed, n):
    """n extension-field elements drawn like SplitMix.elem_ext (no rejection
    can occur in practice; asserted)."""
    v = splitmix_words(seed, 2 * n) >> np.uint64(3)
    assert not np.any(v == np.uint64((1 << 61) - 1))
    return v.reshape(n, 2).copy()


def splitmix_base(seed, n):
    v = splitmix_words(seed, n) >> np.uint64(3)
    assert not np.any(v == np.uint64((1 << 61) - 1))
    out = np.zeros((n, 2), dtype=np.uint64)
    out[:, 0] = v
    return out


def batch_open_inputs(oracle, rate, whir_k, seed, logs):
    """Inputs of a Whir_Batch_Open case as the reference driver builds them
    (oracle/ref/ref_full_driver.cpp cmd_batchopen): arrays, then one point
    per array from the same SplitMix stream; betas = eq tables of the points;
    K0 = <arrays[0], betas[0]>; codewords = RS encodings at the rate each
    array is merged at; levels0 = the Merkle tree of codeword 0."""
    n = [1 << l for l in logs]
    raw = splitmix_ext(seed, sum(n) + sum(logs))
    arrays, off = [], 0
    for x in n:
        arrays.append(raw[off:off + x])
        off += x
    betas = []
    for l in logs:
        betas.append(oracle.precompute_beta(raw[off:off + l]))
        off += l
    sch = oracle.whir_batch_schedule(n, rate, whir_k)
    assert sch is not None
    cws = []
    for a, L in zip(arrays, sch[2]):
        if L == 0:
            cws.append(None)
            continue
        c = np.zeros((L, 2), dtype=np.uint64)
        c[:a.shape[0]] = a
        cws.append(oracle.fft(c))
    levels0 = oracle.merkle_commit(cws[0])
    _, _, K0 = oracle.aggregate_arrays(np.zeros_like(arrays[0]), np.zeros_like(betas[0]), [arrays[0]], [betas[0]],
                                       [[1, 0]], [[1, 0]])
    return arrays, betas, cws, levels0, K0, sch
