"""NTT shape autotuning: every candidate four-step shape gives the same
transform (exact arithmetic), and the tuner installs a valid shape."""
import numpy as np
import pytest

from conftest import rand_fe

pytestmark = pytest.mark.gpu


def candidates(logn):
    out = []
    for k1 in range(1, 14):
        k2 = logn - k1
        if not 1 <= k2 <= 13 or abs(k1 - k2) > 2:
            continue
        for a in range(0, min(k1, 13 - k2) + 1):
            for b in range(0, min(k2, 13 - k1) + 1):
                if (a == 0 and k2 < 13) or a > 4 or b > 3:
                    continue
                out.append((k1, a, b))
    return out


@pytest.mark.parametrize("logn", [14, 17, 20])
def test_every_shape_same_transform(ctx, gbz, oracle, logn):
    rng = np.random.default_rng(logn)
    x = rand_fe(rng, 1 << logn)
    ref_f = oracle.fft(x.copy(), False)
    ref_i = oracle.fft(x.copy(), True)
    saved = gbz.ntt_get_shape(logn)
    try:
        for sh in candidates(logn):
            gbz.ntt_set_shape(logn, *sh)
            assert np.array_equal(ctx.fft(x.copy(), logn, False), ref_f), sh
            assert np.array_equal(ctx.fft(x.copy(), logn, True), ref_i), sh
    finally:
        gbz.ntt_set_shape(logn, *saved)


def test_autotune_installs_valid_shape(ctx, gbz, oracle):
    logn = 18
    saved = gbz.ntt_get_shape(logn)
    try:
        shape, ms_def, ms_best = ctx.ntt_autotune(logn, reps=2)
        assert gbz.ntt_get_shape(logn) == shape
        assert 0 < ms_best <= ms_def
        rng = np.random.default_rng(3)
        x = rand_fe(rng, 1 << logn)
        assert np.array_equal(ctx.fft(x.copy(), logn, False), oracle.fft(x.copy(), False))
    finally:
        gbz.ntt_set_shape(logn, *saved)


def test_invalid_shape_rejected(gbz):
    with pytest.raises(gbz.GbzError):
        gbz.ntt_set_shape(20, 13, 7, 0)   # first pass would stage 2^(7+7) > 2^13 elements
    with pytest.raises(gbz.GbzError):
        gbz.ntt_set_shape(20, 6, 0, 0)    # first pass of length 2^14 does not fit one CTA
    with pytest.raises(gbz.GbzError):
        gbz.ntt_set_shape(12, 6, 1, 1)    # lengths up to 2^13 take one pass


@pytest.mark.parametrize("logN", [2, 5, 13, 14, 15, 24, 26])
def test_merkle_fusion_depths_same_tree(ctx, gbz, oracle, logN):
    rng = np.random.default_rng(logN)
    x = rand_fe(rng, 1 << logN)
    ref = None if logN > 20 else oracle.merkle_commit(x)
    saved = gbz.lib.gbz_merkle_get_fusion()
    got = {}
    try:
        for lg in (10, 11):
            assert gbz.lib.gbz_merkle_set_fusion(lg) == gbz.OK
            got[lg] = ctx.merkle_commit_flat(x)
    finally:
        gbz.lib.gbz_merkle_set_fusion(saved)
    assert np.array_equal(got[10], got[11])
    if ref is not None:
        assert np.array_equal(got[10].reshape(-1), np.asarray(ref).reshape(-1))


def test_merkle_autotune(ctx, gbz):
    saved = gbz.lib.gbz_merkle_get_fusion()
    try:
        lg, ms_def, ms_best = ctx.merkle_autotune(20, reps=2)
        assert lg in (10, 11) and gbz.lib.gbz_merkle_get_fusion() == lg and ms_best <= ms_def
    finally:
        gbz.lib.gbz_merkle_set_fusion(saved)
    assert gbz.lib.gbz_merkle_set_fusion(12) == gbz.EINVAL


@pytest.mark.parametrize("logn", [14, 19, 23])
def test_full_twiddle_tables_same_transform(ctx, gbz, oracle, logn):
    rng = np.random.default_rng(100 + logn)
    x = rand_fe(rng, 1 << logn)
    try:
        gbz.lib.gbz_ntt_full_twiddles(0)
        f0, i0 = ctx.fft(x.copy(), logn, False), ctx.fft(x.copy(), logn, True)
    finally:
        gbz.lib.gbz_ntt_full_twiddles(1)
    f1, i1 = ctx.fft(x.copy(), logn, False), ctx.fft(x.copy(), logn, True)
    assert np.array_equal(f0, f1) and np.array_equal(i0, i1)
    if logn <= 19:
        assert np.array_equal(f1, oracle.fft(x.copy(), False))
