"""The oracle's Whir_Batch_Open (oracle/gbz_oracle.c orc_whir_batch_open)
against transcripts of the reference (ref_full batchopen), and its schedule
checks.  CPU only."""
import hashlib

import numpy as np
import pytest

from conftest import batch_open_inputs, golden_bytes


def oracle_transcript(oracle, args):
    rate, whir_k, seed, prng = args[:4]
    arrays, betas, cws, levels0, K0, _ = batch_open_inputs(oracle, rate, whir_k, seed, args[4:])
    t, ok, g = oracle.whir_batch_open(arrays, cws, levels0, betas, K0, rate, whir_k, prng_seed=prng)
    assert ok, "final claim differs from sum arr * b"
    return t + np.int32(g.next()).tobytes()


def test_batch_open_golden_full(oracle, golden):
    e = golden["batchopen"]["bo_7_5_r16"]
    assert oracle_transcript(oracle, e["args"]) == golden_bytes(e["file"])


@pytest.mark.parametrize("name", ["bo_8_8_r8", "bo_9_7_7_r4", "bo_10_8_6_r8", "bo_10_9_r4", "bo_9_6_r8_k2",
                                  "bo_10_7_r4_k8", "bo_12_10_10_7_r2", "bo_13_9_9_9_6_r2", "bo_16_12_10_r2"])
def test_batch_open_golden_digest(oracle, golden, name):
    e = golden["batchopen"][name]
    t = oracle_transcript(oracle, e["args"])
    assert len(t) == e["bytes"]
    assert hashlib.sha256(t).hexdigest() == e["sha256"]


def test_batch_schedule(oracle):
    kap, agg, cwl, nb = oracle.whir_batch_schedule([1 << 12, 1 << 10, 1 << 10, 1 << 7], 2, 4)
    assert (kap, agg) == ([4, 4, 2, 4, 4, 4], [1, 0, 1, 0, 0, 0])
    assert cwl == [8192, 4096, 4096, 2048]
    # equal sizes first: merged before any iteration (kappa 1)
    assert oracle.whir_batch_schedule([256, 256], 8, 4)[:2] == ([1, 4, 4, 4], [1, 0, 0, 0])


@pytest.mark.parametrize("sizes,rate,whir_k", [
    ([1 << 11, 1 << 8, 4], 4, 4),   # merge at the last schedule step: the reference reads kappas past its end
    ([1 << 12, 1 << 8], 2, 16),
    ([64, 128], 2, 4),              # sizes must not increase
    ([96], 2, 4),                   # not a power of two
    ([1 << 10], 2, 3),              # whir_k must be 2, 4, 8 or 16
    ([1 << 10], 3, 4),              # rate must be a power of two >= 2
    ([4], 2, 4),                    # shorter than 2 whir_k
])
def test_batch_schedule_rejects(oracle, sizes, rate, whir_k):
    assert oracle.whir_batch_schedule(sizes, rate, whir_k) is None
