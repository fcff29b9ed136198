"""GPU WHIR aggregation (aggregate_claims / aggregate_arrays /
aggregate_commitments) against the reference fixtures and the oracle."""
import numpy as np
import pytest

from conftest import rand_fe
from test_oracle_sumcheck import case
from test_oracle_whir_aggr import arrays_inputs, claims_inputs, commit_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["aggclaims_6_2_3", "aggclaims_9_4_2", "aggclaims_5_1_1"])
def test_aggregate_claims_golden(ctx, golden, name):
    r, args = case(golden, name)
    n, k, c, arrays, points, prng = claims_inputs(args)
    arr, b, K, bch, ach = r.fe(n), r.fe(n), r.fe(1)[0], r.fe(c), r.fe(k)
    garr, gb, gK, gch, _, _ = ctx.aggregate_claims(arrays, points, prng=prng)
    assert np.array_equal(garr, arr)
    assert np.array_equal(gb, b)
    assert np.array_equal(gK, K)
    assert np.array_equal(gch, np.concatenate([bch, ach]))


@pytest.mark.parametrize("k,c,logn", [(1, 1, 3), (5, 7, 12), (9, 2, 16), (3, 3, 20), (4, 4, 13), (2, 1, 2),
                                        (4, 2, 1)])
def test_aggregate_claims_vs_oracle(ctx, oracle, k, c, logn):
    rng = np.random.default_rng(300 + k * 10 + c)
    n = 1 << logn
    arrays = [rand_fe(rng, n) for _ in range(k)]
    points = rand_fe(rng, c * logn).reshape(c, logn, 2)
    oarr, ob, oK, och, osums = oracle.aggregate_claims(arrays, points, prng_seed=5)
    garr, gb, gK, gch, gsums, _ = ctx.aggregate_claims(arrays, points, prng=5)
    assert np.array_equal(gsums, osums)
    assert np.array_equal(gch, och)
    assert np.array_equal(gK, oK)
    assert np.array_equal(garr, oarr)
    assert np.array_equal(gb, ob)


@pytest.mark.parametrize("name", ["aggarrays_6_3", "aggarrays_8_2"])
def test_aggregate_arrays_golden(ctx, golden, name):
    r, args = case(golden, name)
    n, k, arrays, B, r1, r2 = arrays_inputs(args)
    arr, b, K = r.fe(n), r.fe(n), r.fe(1)[0]
    garr, gb, gK = ctx.aggregate_arrays(arrays[0], B[0], arrays, B, r1, r2)
    assert np.array_equal(garr, arr)
    assert np.array_equal(gb, b)
    assert np.array_equal(gK, K)


@pytest.mark.parametrize("k,nB,logn", [(1, 1, 4), (3, 6, 13), (8, 8, 18)])
def test_aggregate_arrays_vs_oracle(ctx, oracle, k, nB, logn):
    rng = np.random.default_rng(400 + k + nB)
    n = 1 << logn
    arrays = [rand_fe(rng, n) for _ in range(k)]
    B = [rand_fe(rng, n) for _ in range(nB)]
    r1, r2 = rand_fe(rng, k), rand_fe(rng, nB)
    a0, b0 = rand_fe(rng, n), rand_fe(rng, n)
    ref = oracle.aggregate_arrays(a0, b0, arrays, B, r1, r2)
    got = ctx.aggregate_arrays(a0, b0, arrays, B, r1, r2)
    for g, o in zip(got, ref):
        assert np.array_equal(g, o)


@pytest.mark.parametrize("name", ["aggcommit_8_3_2_4", "aggcommit_10_2_4_8", "aggcommit_7_4_8_4"])
def test_aggregate_commitments_golden(ctx, golden, name):
    r, args = case(golden, name)
    n, k, rate, whir_k, cws, rr, prng = commit_inputs(args)
    cw = r.fe(n)
    leaves = n // whir_k
    levels = np.frombuffer(r.raw(32 * (2 * leaves - 1)), dtype=np.uint8).reshape(-1, 32)
    nxt = np.frombuffer(r.raw(4), dtype=np.int32)[0]
    gcw, glv, g = ctx.aggregate_commitments(cws, rr, rate, whir_k, prng=prng)
    assert np.array_equal(gcw, cw)
    assert np.array_equal(glv, levels)
    assert g.next() == nxt


def test_aggregate_commitments_large(ctx, oracle):
    rng = np.random.default_rng(8)
    n = 1 << 20
    cws = [rand_fe(rng, n) for _ in range(4)]
    r = rand_fe(rng, 4)
    ocw, olv, og = oracle.aggregate_commitments(cws, r, 2, 4, prng_seed=9)
    gcw, glv, gg = ctx.aggregate_commitments(cws, r, 2, 4, prng=9)
    assert np.array_equal(gcw, ocw)
    assert np.array_equal(glv, olv)
    assert gg.next() == og.next()


@pytest.mark.parametrize("name", ["tensor_6_8_2_3", "tensor_9_16_4_0", "tensor_4_4_8_1"])
def test_tensor_eval_vector_golden(ctx, golden, name):
    r, (_, logrows, N, rate, my_id, p0, p1) = case(golden, name)
    B = r.fe(1 << logrows)
    assert np.array_equal(ctx.tensor_eval_vector((p0, p1), N // 2, 1 << logrows, rate, my_id), B)


@pytest.mark.parametrize("name", ["phase3_6_8_3_2_1", "phase3_10_16_20_4_5", "phase3_8_64_7_2_63"])
def test_pcs_phase3_golden(ctx, golden, name):
    from test_oracle_whir_aggr import phase3_inputs
    r, args = case(golden, name)
    rows, N, l, rate, my_id, B0, s, q = phase3_inputs(r, args)
    B = r.fe(rows)
    assert np.array_equal(ctx.pcs_sumcheck_phase3(B0, q, s, N, rate, my_id), B)


@pytest.mark.parametrize("logrows,N,l,rate", [(14, 16, 100, 2), (18, 4, 300, 4), (20, 16, 50, 2)])
def test_pcs_phase3_vs_oracle(ctx, oracle, logrows, N, l, rate):
    """Includes the sparse-transform path (l rows above a few transform
    lengths) and more than 256 queries (chunked)."""
    rng = np.random.default_rng(logrows + N + l)
    rows = 1 << logrows
    B0 = rand_fe(rng, rows)
    s = rand_fe(rng, 1)[0]
    q = np.stack([rng.integers(0, N // 2, size=l), rng.integers(0, rate * rows, size=l)], axis=1).astype(np.uint32)
    my_id = int(rng.integers(0, N))
    assert np.array_equal(ctx.pcs_sumcheck_phase3(B0, q, s, N, rate, my_id),
                          oracle.pcs_phase3(B0, q, s, N, rate, my_id))
