"""gbz_whir_batch_schedule (host only) equals the oracle's restatement of
Whir_Batch_Open's schedule over a sweep of size lists.  CPU only."""
import itertools

import pytest


def size_lists():
    for n0 in (3, 4, 6, 9, 12, 16):
        for extra in itertools.chain([()], itertools.combinations_with_replacement(range(1, n0 + 1), 1),
                                     itertools.combinations_with_replacement(range(2, n0 + 1, 2), 2)):
            yield [1 << n0] + sorted((1 << e for e in extra), reverse=True)


@pytest.mark.parametrize("rate,whir_k", [(2, 4), (4, 4), (8, 2), (2, 8), (16, 16), (3, 4), (2, 5)])
def test_schedule_matches_oracle(gbz, oracle, rate, whir_k):
    n = 0
    for sizes in size_lists():
        a = gbz.whir_batch_schedule(sizes, rate, whir_k)
        b = oracle.whir_batch_schedule(sizes, rate, whir_k)
        assert a == b, sizes
        n += a is not None
    if rate in (2, 4, 8, 16) and whir_k in (2, 4, 8, 16):
        assert n > 0
