"""Whir_Batch_Open on the GPU (gbz_whir_batch_open) against the reference's
transcripts and the oracle."""
import hashlib

import numpy as np
import pytest

from conftest import batch_open_inputs, golden_bytes

pytestmark = pytest.mark.gpu

GOLDEN = ["bo_7_5_r16", "bo_8_8_r8", "bo_9_7_7_r4", "bo_10_8_6_r8", "bo_10_9_r4", "bo_9_6_r8_k2",
          "bo_10_7_r4_k8", "bo_12_10_10_7_r2", "bo_13_9_9_9_6_r2", "bo_16_12_10_r2"]


def gpu_transcript(ctx, oracle, args, mem="host"):
    rate, whir_k, seed, prng = args[:4]
    arrays, betas, cws, levels0, K0, _ = batch_open_inputs(oracle, rate, whir_k, seed, args[4:])
    if mem == "device":
        import torch
        dev = lambda x: None if x is None else torch.from_numpy(x.view(np.int64)).cuda()
        arrays, betas, cws = [dev(a) for a in arrays], [dev(b) for b in betas], [dev(c) for c in cws]
        levels0 = torch.from_numpy(levels0).cuda()
    t, g = ctx.whir_batch_open(arrays, cws, levels0, betas, K0, rate, whir_k, prng=prng)
    if mem == "device":
        t = t.cpu().numpy()
    return t.tobytes() + np.int32(g.next()).tobytes()


@pytest.mark.parametrize("name", GOLDEN)
def test_batch_open_vs_reference(ctx, oracle, golden, name):
    e = golden["batchopen"][name]
    t = gpu_transcript(ctx, oracle, e["args"])
    if "file" in e:
        assert t == golden_bytes(e["file"])
    assert len(t) == e["bytes"]
    assert hashlib.sha256(t).hexdigest() == e["sha256"]


@pytest.mark.parametrize("args", [
    (2, 4, 201, 1, 11, 9), (4, 4, 202, 7, 12, 12, 10), (8, 2, 203, 3, 10, 8, 8, 8), (2, 8, 204, 1, 13, 10),
    (16, 4, 205, 2, 9, 9, 9, 7), (2, 4, 206, 4, 14, 12, 10, 8), (4, 16, 207, 1, 14, 10),
])
def test_batch_open_vs_oracle(ctx, oracle, args):
    rate, whir_k, seed, prng = args[:4]
    if oracle.whir_batch_schedule([1 << l for l in args[4:]], rate, whir_k) is None:
        pytest.skip("the reference cannot run these sizes")
    arrays, betas, cws, levels0, K0, _ = batch_open_inputs(oracle, rate, whir_k, seed, args[4:])
    ref, ok, g = oracle.whir_batch_open(arrays, cws, levels0, betas, K0, rate, whir_k, prng_seed=prng)
    assert ok
    got, g2 = ctx.whir_batch_open(arrays, cws, levels0, betas, K0, rate, whir_k, prng=prng)
    assert got.tobytes() == ref
    assert g2.next() == g.next()


def test_batch_open_device_buffers(ctx, oracle, golden):
    e = golden["batchopen"]["bo_10_8_6_r8"]
    t = gpu_transcript(ctx, oracle, e["args"], mem="device")
    assert hashlib.sha256(t).hexdigest() == e["sha256"]


def test_batch_open_wrong_claim_is_flagged(ctx, oracle, gbz):
    arrays, betas, cws, levels0, K0, _ = batch_open_inputs(oracle, 4, 4, 301, (10, 8))
    bad = np.array(K0, dtype=np.uint64)
    bad[0] = (int(bad[0]) + 1) % ((1 << 61) - 1)
    with pytest.raises(gbz.GbzError) as ei:
        ctx.whir_batch_open(arrays, cws, levels0, betas, bad, 4, 4, prng=1)
    assert ei.value.status == gbz.ECHECK
    # the context stays usable
    t, _ = ctx.whir_batch_open(arrays, cws, levels0, betas, K0, 4, 4, prng=1)
    ref, ok, _ = oracle.whir_batch_open(arrays, cws, levels0, betas, K0, 4, 4, prng_seed=1)
    assert ok and t.tobytes() == ref


def test_batch_open_rejects_unrunnable(ctx, oracle, gbz):
    arrays = [np.zeros((1 << 11, 2), np.uint64), np.zeros((1 << 8, 2), np.uint64), np.zeros((4, 2), np.uint64)]
    with pytest.raises(gbz.GbzError) as ei:
        ctx.whir_batch_open(arrays, [None] * 3, np.zeros((1, 32), np.uint8), arrays, [0, 0], 4, 4)
    assert ei.value.status == gbz.EINVAL
