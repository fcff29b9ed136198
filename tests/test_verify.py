"""The standalone transcript verifier (gbz_verify_proof, host code) on the
oracle's transcripts, which equal the reference prover's byte for byte
(tests/test_oracle_golden.py pins them): every honest transcript passes,
and each planted change in a copy of one is caught by the check that
covers it.  The changes are made in the oracle's transcript on the CPU."""
import numpy as np
import pytest

SHAPES = [(3, 2), (4, 4), (7, 2), (10, 4), (11, 8), (12, 2), (13, 16)]


def transcript(oracle, logn, rate, seed):
    w = oracle.witness(0x7E57 + logn * 131 + rate, 1 << logn)
    return bytearray(oracle.prove(w, logn, rate, seed))


@pytest.mark.parametrize("logn,rate", SHAPES)
def test_honest_transcripts_verify(gbz, oracle, logn, rate):
    for seed in (1, 7):
        ok, failed = gbz.verify_proof(transcript(oracle, logn, rate, seed), logn, rate, seed)
        assert ok and failed == [], (logn, rate, seed, failed)


def records(gbz, tr):
    """[(tag, payload offset, count)] of a transcript."""
    out, off = [], 0
    for tag, count, payload in gbz.parse_transcript(bytes(tr)):
        out.append((tag, off + 8, count))
        off += 8 + len(payload)
    return out


def flip(tr, off):
    tr[off] ^= 1


@pytest.mark.parametrize("tag,check", [(2, "point"), (4, "sumcheck_sum"), (5, "sumcheck_challenge"),
                                       (6, "sumcheck_final"), (7, "whir_sum"), (8, "whir_challenge"),
                                       (10, "queries"), (12, "answers"), (14, "combine"), (15, "whir_K"),
                                       (17, "final_point"), (16, "step2"), (18, "step3")])
def test_tampering_is_caught(gbz, oracle, tag, check):
    logn, rate, seed = 10, 4, 3
    tr = transcript(oracle, logn, rate, seed)
    off = next(o for t, o, c in records(gbz, tr) if t == tag)
    flip(tr, off)
    ok, failed = gbz.verify_proof(tr, logn, rate, seed)
    assert not ok and check in failed, (tag, failed)


def test_reply_change_breaks_its_answer(gbz, oracle):
    logn, rate, seed = 9, 2, 5
    tr = transcript(oracle, logn, rate, seed)
    off = next(o for t, o, c in records(gbz, tr) if t == 11)
    flip(tr, off + 16 * 4)              # second query's first reply
    ok, failed = gbz.verify_proof(tr, logn, rate, seed)
    assert not ok and failed == ["answers"]


def test_wrong_seed_or_shape_fails(gbz, oracle):
    logn, rate = 8, 4
    tr = transcript(oracle, logn, rate, 1)
    ok, failed = gbz.verify_proof(tr, logn, rate, 2)
    assert not ok and "whir_challenge" in failed
    ok, failed = gbz.verify_proof(tr, logn + 1, rate, 1)
    assert not ok and "layout" in failed
    ok, failed = gbz.verify_proof(tr[:-16], logn, rate, 1)
    assert not ok and "layout" in failed
