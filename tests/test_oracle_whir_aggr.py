"""The oracle's WHIR aggregation functions (aggregate_claims,
aggregate_arrays, aggregate_commitments) against the reference's outputs.
CPU only."""
import numpy as np
import pytest

from conftest import splitmix_ext
from test_oracle_sumcheck import case


def claims_inputs(args):
    _, logn, k, c, seed, prng = args
    n = 1 << logn
    raw = splitmix_ext(seed, k * n + c * logn)
    arrays = [raw[i * n:(i + 1) * n] for i in range(k)]
    points = raw[k * n:].reshape(c, logn, 2)
    return n, k, c, arrays, points, prng


def arrays_inputs(args):
    _, logn, k, seed = args
    n = 1 << logn
    raw = splitmix_ext(seed, 2 * k * n + 2 * k)
    arrays = [raw[i * n:(i + 1) * n] for i in range(k)]
    B = [raw[(k + i) * n:(k + i + 1) * n] for i in range(k)]
    r1, r2 = raw[2 * k * n:2 * k * n + k], raw[2 * k * n + k:]
    return n, k, arrays, B, r1, r2


def commit_inputs(args):
    _, logn, k, rate, whir_k, seed, prng = args
    n = 1 << logn
    raw = splitmix_ext(seed, k * n + k)
    return n, k, rate, whir_k, [raw[i * n:(i + 1) * n] for i in range(k)], raw[k * n:], prng


@pytest.mark.parametrize("name", ["aggclaims_6_2_3", "aggclaims_9_4_2", "aggclaims_5_1_1"])
def test_aggregate_claims(oracle, golden, name):
    r, args = case(golden, name)
    n, k, c, arrays, points, prng = claims_inputs(args)
    arr, b, K, bch, ach = r.fe(n), r.fe(n), r.fe(1)[0], r.fe(c), r.fe(k)
    r.done()
    garr, gb, gK, gch, _ = oracle.aggregate_claims(arrays, points, prng_seed=prng)
    assert np.array_equal(garr, arr)
    assert np.array_equal(gb, b)
    assert np.array_equal(gK, K)
    assert np.array_equal(gch[:c], bch)
    assert np.array_equal(gch[c:], ach)


@pytest.mark.parametrize("name", ["aggarrays_6_3", "aggarrays_8_2"])
def test_aggregate_arrays(oracle, golden, name):
    r, args = case(golden, name)
    n, k, arrays, B, r1, r2 = arrays_inputs(args)
    arr, b, K = r.fe(n), r.fe(n), r.fe(1)[0]
    r.done()
    garr, gb, gK = oracle.aggregate_arrays(arrays[0], B[0], arrays, B, r1, r2)
    assert np.array_equal(garr, arr)
    assert np.array_equal(gb, b)
    assert np.array_equal(gK, K)


@pytest.mark.parametrize("name", ["aggcommit_8_3_2_4", "aggcommit_10_2_4_8", "aggcommit_7_4_8_4"])
def test_aggregate_commitments(oracle, golden, name):
    r, args = case(golden, name)
    n, k, rate, whir_k, cws, rr, prng = commit_inputs(args)
    cw = r.fe(n)
    leaves = n // whir_k
    levels = np.frombuffer(r.raw(32 * (2 * leaves - 1)), dtype=np.uint8).reshape(-1, 32)
    nxt = np.frombuffer(r.raw(4), dtype=np.int32)[0]
    r.done()
    gcw, glv, g = oracle.aggregate_commitments(cws, rr, rate, whir_k, prng_seed=prng)
    assert np.array_equal(gcw, cw)
    assert np.array_equal(glv, levels)
    assert g.next() == nxt


@pytest.mark.parametrize("name", ["tensor_6_8_2_3", "tensor_9_16_4_0", "tensor_4_4_8_1"])
def test_tensor_eval_vector(oracle, golden, name):
    r, (_, logrows, N, rate, my_id, p0, p1) = case(golden, name)
    B = r.fe(1 << logrows)
    r.done()
    assert np.array_equal(oracle.tensor_eval_vector((p0, p1), N // 2, 1 << logrows, rate, my_id), B)


def phase3_inputs(r, args):
    _, logrows, N, l, rate, my_id, seed = args
    rows = 1 << logrows
    raw = splitmix_ext(seed, rows + 1)
    q = np.frombuffer(r.raw(8 * l), dtype=np.uint32).reshape(l, 2)
    return rows, N, l, rate, my_id, raw[:rows], raw[rows], q


@pytest.mark.parametrize("name", ["phase3_6_8_3_2_1", "phase3_10_16_20_4_5", "phase3_8_64_7_2_63"])
def test_pcs_phase3(oracle, golden, name):
    r, args = case(golden, name)
    rows, N, l, rate, my_id, B0, s, q = phase3_inputs(r, args)
    B = r.fe(rows)
    r.done()
    assert np.array_equal(oracle.pcs_phase3(B0, q, s, N, rate, my_id), B)


@pytest.mark.parametrize("name", ["encconc_8_2_2_4", "encconc_10_4_2_16", "encconc_6_2_4_8"])
def test_encode_concatenated(oracle, golden, name):
    r, (_, logn, rate0, rate1, degree, seed) = case(golden, name)
    n = 1 << logn
    L = n * rate0
    Cp = r.fe(L)
    C = np.stack([r.fe(degree * rate1) for _ in range(L // degree)])
    r.done()
    gCp, gC = oracle.encode_concatenated(splitmix_ext(seed, n), rate0, rate1, degree)
    assert np.array_equal(gCp, Cp)
    assert np.array_equal(gC, C)
