"""Whir_Open on caller arrays (gbz_whir_open) against the opening inside a
whole proof (gbz_prove, whose transcripts equal the reference's fixtures):
the same witness, its codeword, the sumcheck's challenges as the point and
its final value as the claim, and the same glibc stream give the same
commitment root and WHIR records byte for byte."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T_COMMIT_ROOT, T_SC_CHALLENGE, T_SC_FINAL, T_WHIR_POLY = 1, 5, 6, 7


@pytest.mark.parametrize("logn,rate,seed", [(10, 4, 1), (13, 2, 7), (16, 2, 3), (12, 8, 5)])
def test_open_equals_the_proof_opening(gbz, oracle, ctx, logn, rate, seed):
    w = oracle.witness(0x5EED7000 + logn, 1 << logn)
    full = gbz.parse_transcript(ctx.prove(w, logn, rate, seed).tobytes())
    chal = np.array([np.frombuffer(p, dtype=np.uint64) for t, c, p in full if t == T_SC_CHALLENGE])
    K = np.frombuffer([p for t, c, p in full if t == T_SC_FINAL][0][:16], dtype=np.uint64)
    cw = ctx.rs_encode(w, rate)
    g = gbz.Prng(seed)
    tr = gbz.parse_transcript(ctx.Whir_Open(w, logn, rate, cw, chal, K, g))
    first = next(i for i, r in enumerate(full) if r[0] == T_WHIR_POLY)
    assert tr[0] == full[0] and tr[0][0] == T_COMMIT_ROOT
    assert tr[1:] == full[first:]
    # the generator moved past the opening's draws, as the reference's does
    assert g.next() != gbz.Prng(seed).next()


def test_wrong_claim_is_rejected(gbz, oracle, ctx):
    logn, rate = 10, 4
    w = oracle.witness(0x5EED7000 + logn, 1 << logn)
    full = gbz.parse_transcript(ctx.prove(w, logn, rate, 1).tobytes())
    chal = np.array([np.frombuffer(p, dtype=np.uint64) for t, c, p in full if t == T_SC_CHALLENGE])
    K = np.frombuffer([p for t, c, p in full if t == T_SC_FINAL][0][:16], dtype=np.uint64).copy()
    K[0] ^= 1
    with pytest.raises(gbz.GbzError) as e:
        ctx.Whir_Open(w, logn, rate, ctx.rs_encode(w, rate), chal, K, gbz.Prng(1))
    assert e.value.status == gbz.ECHECK


@pytest.mark.parametrize("logL", [1, 2, 5, 12])
def test_tree_from_leaves_equals_commit_levels(gbz, oracle, ctx, logL):
    """create_tree_blake over the leaf level of a reference Merkle commit
    rebuilds the commit's upper levels."""
    rng = np.random.default_rng(logL)
    elems = rng.integers(0, (1 << 61) - 1, size=(4 << logL, 2), dtype=np.uint64)
    levels = oracle.merkle_commit(elems)
    L = 1 << logL
    assert np.array_equal(ctx.create_tree_blake(levels[:L]), levels[L:])
