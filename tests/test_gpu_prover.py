"""GPU prover: transcripts bit-identical to the oracle and to the reference.

The golden digests at 2^18 (rate 1/4) and 2^24 (rate 1/2) are the
reference's own transcripts for the two plain-prover workloads.
"""
import ctypes
import hashlib

import numpy as np
import pytest

from conftest import golden_bytes, splitmix_base

pytestmark = pytest.mark.gpu


def _cudart():
    rt = ctypes.CDLL("libcudart.so")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return rt


@pytest.mark.parametrize("logn,rate,prng_seed", [
    (3, 2, 1), (4, 2, 1), (4, 4, 3), (5, 2, 1), (5, 8, 2), (6, 4, 1), (7, 2, 9), (8, 4, 1), (9, 2, 1),
    (10, 4, 77), (11, 2, 1), (12, 8, 1), (13, 2, 5), (14, 4, 1), (15, 2, 1), (16, 4, 123),
])
def test_prove_vs_oracle(ctx, oracle, logn, rate, prng_seed):
    w = oracle.witness(1000 + logn, 1 << logn)
    got = ctx.prove(w, logn, rate, prng_seed).tobytes()
    ref = oracle.prove(w, logn, rate, prng_seed)
    if got != ref:
        import gbz
        a, b = gbz.parse_transcript(got), gbz.parse_transcript(ref)
        for k, (x, y) in enumerate(zip(a, b)):
            assert x == y, "first differing record %d: tag %d" % (k, y[0])
    assert got == ref


def test_prove_golden_full(ctx, golden):
    e = golden["prove"][0]
    w = splitmix_base(e["seed"], 1 << e["logn"])
    assert ctx.prove(w, e["logn"], e["rate"], e["prng_seed"]).tobytes() == golden_bytes(e["file"])


@pytest.mark.parametrize("idx", range(1, 11))
def test_prove_golden_digests(ctx, golden, idx):
    """Includes the reference transcripts of 2^18 at rate 4 and 2^24 at rate 2."""
    e = golden["prove"][idx]
    w = splitmix_base(e["seed"], 1 << e["logn"])
    t = ctx.prove(w, e["logn"], e["rate"], e["prng_seed"]).tobytes()
    assert len(t) == e["bytes"]
    assert hashlib.sha256(t).hexdigest() == e["sha256"]


def test_prove_repeatable_and_seed_sensitive(ctx, oracle):
    w = oracle.witness(5, 1 << 12)
    a = ctx.prove(w, 12, 4, 1).tobytes()
    b = ctx.prove(w, 12, 4, 1).tobytes()
    c = ctx.prove(w, 12, 4, 2).tobytes()
    assert a == b
    assert a != c
    # same shape, other witness, then the first again: no state leaks between proofs
    ctx.prove(oracle.witness(6, 1 << 12), 12, 4, 1)
    assert ctx.prove(w, 12, 4, 1).tobytes() == a


def test_prove_device_pointers(ctx, gbz, oracle):
    """Witness and transcript in device memory (GBZ_MEM_DEVICE)."""
    logn, rate = 14, 2
    w = oracle.witness(31, 1 << logn)
    nbytes = gbz.transcript_bytes(logn, rate)
    rt = _cudart()
    dw, dt = ctypes.c_void_p(), ctypes.c_void_p()
    ctx.check(gbz.lib.gbz_device_alloc(ctx.h, ctypes.byref(dw), w.nbytes))
    ctx.check(gbz.lib.gbz_device_alloc(ctx.h, ctypes.byref(dt), nbytes))
    try:
        assert rt.cudaMemcpy(dw, w.ctypes.data, w.nbytes, 1) == 0
        ctx.check(gbz.lib.gbz_prove(ctx.h, dw, logn, rate, 1, dt, nbytes, gbz.MEM_DEVICE))
        ctx.synchronize()
        out = np.zeros(nbytes, dtype=np.uint8)
        assert rt.cudaMemcpy(out.ctypes.data, dt, nbytes, 2) == 0
        assert out.tobytes() == oracle.prove(w, logn, rate, 1)
    finally:
        gbz.lib.gbz_device_free(ctx.h, dw)
        gbz.lib.gbz_device_free(ctx.h, dt)


def test_prove_small_buffer_rejected(ctx, gbz, oracle):
    w = oracle.witness(1, 1 << 8)
    out = np.zeros(gbz.transcript_bytes(8, 4) - 1, dtype=np.uint8)
    with pytest.raises(gbz.GbzError) as e:
        ctx.prove(w, 8, 4, 1, out=out)
    assert e.value.status == gbz.ESMALL


def test_two_contexts_interleaved(gbz, oracle):
    """Independent contexts (one stream each) give the same transcripts."""
    c1, c2 = gbz.Context(0), gbz.Context(0)
    try:
        w1, w2 = oracle.witness(71, 1 << 13), oracle.witness(72, 1 << 13)
        t1 = c1.prove(w1, 13, 2, 1).tobytes()
        t2 = c2.prove(w2, 13, 2, 4).tobytes()
        assert t1 == oracle.prove(w1, 13, 2, 1)
        assert t2 == oracle.prove(w2, 13, 2, 4)
    finally:
        c1.close()
        c2.close()


def test_prove_graph_replay_matches_direct_launches(ctx, oracle):
    """gbz_prove replays a captured graph by default; the seed is a graph
    parameter, so seeds and witnesses change freely between replays."""
    w = oracle.witness(77, 1 << 13)
    ctx.set_graphs(False)
    try:
        direct = [ctx.prove(w, 13, 4, s).tobytes() for s in (1, 2, 3)]
    finally:
        ctx.set_graphs(True)
    replay = [ctx.prove(w, 13, 4, s).tobytes() for s in (1, 2, 3, 1)]
    assert replay[:3] == direct
    assert replay[3] == direct[0]
    assert oracle.prove(w, 13, 4, 2) == direct[1]


def test_prove_graph_per_device_address(ctx, gbz, oracle):
    """More device witness addresses than cached graphs (least recently used
    dropped): every transcript still equals the oracle's."""
    torch = pytest.importorskip("torch")
    logn, rate = 11, 2
    ws = [oracle.witness(500 + k, 1 << logn) for k in range(6)]
    dws = [torch.from_numpy(w.view(np.int64)).cuda() for w in ws]
    tb = gbz.transcript_bytes(logn, rate)
    for rep in range(2):
        for k, dw in enumerate(dws):
            out = torch.zeros(tb, dtype=torch.uint8, device="cuda")
            ctx.prove(dw, logn, rate, 1 + k, out=out)
            torch.cuda.synchronize()
            assert out.cpu().numpy().tobytes() == oracle.prove(ws[k], logn, rate, 1 + k)


@pytest.mark.parametrize("logn,rate,seed", [(25, 2, 3), (20, 64, 5), (18, 32, 1)])
def test_prove_largest_shapes_vs_oracle(ctx, oracle, logn, rate, seed):
    """The largest codewords the prover takes (2^26: a 2^25 witness at rate
    1/2, or 2^20 at rate 1/64) and a high rate, against the oracle."""
    w = oracle.witness(0x5EED0000 + 7 * 65536 + logn, 1 << logn)
    got = ctx.prove(w, logn, rate, seed).tobytes()
    ref = oracle.prove(w, logn, rate, seed)
    assert len(got) == len(ref)
    assert hashlib.sha256(got).hexdigest() == hashlib.sha256(ref).hexdigest()


def test_prove_rejects_out_of_range_shapes(ctx, gbz, oracle):
    w = oracle.witness(2, 1 << 8)
    for logn, rate in ((26, 2), (21, 64), (27, 2), (2, 2), (8, 3), (8, 1), (8, 128)):
        with pytest.raises(gbz.GbzError) as e:
            ctx.prove(np.zeros((1 << min(logn, 8), 2), np.uint64), logn, rate, 1)
        assert e.value.status in (gbz.EINVAL, gbz.ESMALL)


def _extension_witness(seed, n):
    """Canonical F_{p^2} entries with non-zero imaginary words."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, (1 << 61) - 1, size=(n, 2), dtype=np.uint64)


@pytest.mark.parametrize("logn,rate", [(3, 2), (5, 4), (8, 2), (11, 8), (13, 2), (14, 2), (16, 4)])
def test_prove_extension_witness_vs_oracle(ctx, oracle, logn, rate):
    """A witness outside the base field takes the general commit transform
    (the packed real transform flags it) and still matches the oracle."""
    w = _extension_witness(900 + logn, 1 << logn)
    assert ctx.prove(w, logn, rate, 3).tobytes() == oracle.prove(w, logn, rate, 3)


@pytest.mark.parametrize("pos", [0, 1, 4097, (1 << 14) - 1])
def test_prove_single_imaginary_word_then_base_again(ctx, oracle, pos):
    """One non-zero imaginary word anywhere is enough to switch the commit
    to the general transform, and the flag is cleared for the next proof
    replayed on the same buffers."""
    logn, rate = 14, 2
    base = oracle.witness(4242, 1 << logn)
    one = base.copy()
    one[pos, 1] = 12345
    for w in (base, one, base):
        assert ctx.prove(w, logn, rate, 1).tobytes() == oracle.prove(w, logn, rate, 1)
