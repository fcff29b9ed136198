"""The party-share workload at test size: party shares committed and proved on one
device (per-party coPCS Encode + column Merkle + leader root, then the
distributed sumcheck over all parties) equal the oracle's composition of
the same steps."""
import numpy as np
import pytest

from conftest import rand_fe
from test_oracle_sumcheck import fadd, feval

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("P,log_share,rate", [(4, 10, 2), (16, 8, 4)])
def test_party_shares_commit_and_sumcheck(ctx, oracle, P, log_share, rate):
    rng = np.random.default_rng(P * 100 + log_share)
    M, R = 1 << log_share, 16
    n = M // R
    shares = rand_fe(rng, P * M, base=True)
    for p in range(P):
        rows = shares[p * M:(p + 1) * M].reshape(R, n, 2)
        cw = ctx.Encode(rows, rate, 0)
        assert np.array_equal(cw, oracle.encode_rows(rows, rate, 0))
        lv, root = ctx.distributed_MT(cw, P)
        olv, oroot = oracle.column_merkle(cw, P)
        assert np.array_equal(lv, olv)
        assert np.array_equal(root, oroot)
    z = rand_fe(rng, (P * M).bit_length() - 1)
    beta = oracle.precompute_beta(z)
    h = oracle.sumcheck_round(0, [shares, beta])
    y = np.array(fadd(feval(h, (0, 0)), feval(h, (1, 0))), dtype=np.uint64)
    got = ctx.party_sumcheck(0, [shares, beta], P, offset=4, y=y)
    ref = oracle.party_sumcheck(0, [shares, beta], P, offset=4, y=y)
    assert np.array_equal(got["challenges"], ref["challenges"])
    assert np.array_equal(got["fin"], ref["fin"])
