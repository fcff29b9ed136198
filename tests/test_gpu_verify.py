"""gbz_verify_proof on transcripts the GPU prover wrote (gbz_prove, one proof
and a batch of mixed shapes through gbz_prove_batch): all verify."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("logn,rate", [(12, 2), (16, 4), (20, 2), (22, 2)])
def test_gpu_transcripts_verify(gbz, oracle, ctx, logn, rate):
    w = oracle.witness(0x5EED + logn, 1 << logn)
    for seed in (1, 9):
        tr = ctx.prove(w, logn, rate, seed)
        ok, failed = gbz.verify_proof(tr.tobytes(), logn, rate, seed)
        assert ok, (logn, rate, seed, failed)


def test_batch_transcripts_verify(gbz, oracle, ctx):
    logns = [10, 12, 13, 12, 15, 11, 14, 10]
    rates = [4, 2, 4, 8, 2, 4, 2, 16]
    ws = [oracle.witness(0xBA7C + i, 1 << l) for i, l in enumerate(logns)]
    seeds = list(range(3, 3 + len(logns)))
    trs, _, _ = ctx.prove_batch(ws, logns, rates, seeds)
    for t, l, r, s in zip(trs, logns, rates, seeds):
        ok, failed = gbz.verify_proof(t.tobytes(), l, r, s)
        assert ok, (l, r, s, failed)
