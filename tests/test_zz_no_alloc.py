"""gbz_whir_update_betas_noalloc against gbz_whir_update_betas.

The no-allocation entry point serves callers that cannot let the library
allocate device memory during a call (for example a proving service whose
device memory is already divided among request slots).  It must produce the
same beta vector and combination weights as the allocating entry point,
call after call, although every call reuses the same static working array.
This file is collected last so that a failure here does not hide the rest
of the suite in a run that stops at the first failure.
"""
import ctypes

import numpy as np
import pytest

from conftest import rand_fe

pytestmark = pytest.mark.gpu


def _cudart():
    rt = ctypes.CDLL("libcudart.so")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaDeviceSynchronize.argtypes = []
    return rt


class DevBuf:
    def __init__(self, ctx, gbz, host):
        self.ctx, self.gbz, self.nbytes = ctx, gbz, host.nbytes
        self.p = ctypes.c_void_p()
        ctx.check(gbz.lib.gbz_device_alloc(ctx.h, ctypes.byref(self.p), max(self.nbytes, 16)))
        assert _cudart().cudaMemcpy(self.p, host.ctypes.data, self.nbytes, 1) == 0

    def read(self, like):
        out = np.empty_like(like)
        assert _cudart().cudaMemcpy(out.ctypes.data, self.p, self.nbytes, 2) == 0
        return out

    def free(self):
        self.gbz.lib.gbz_device_free(self.ctx.h, self.p)


@pytest.mark.parametrize("logb,logN,l", [(12, 15, 200), (18, 20, 100)])
def test_noalloc_matches_allocating_entry_point_twice(ctx, gbz, logb, logN, l):
    rng = np.random.default_rng(logb + l)
    rt = _cudart()
    for call in range(2):  # two calls in a row share the static working array
        b = rand_fe(rng, 1 << logb)
        q = rng.integers(0, 1 << logN, size=l - 3 * call).astype(np.int32)
        r = rand_fe(rng, 1)[0].copy()
        lq = len(q)
        # existing entry point, device memory
        b1, q1 = DevBuf(ctx, gbz, b), DevBuf(ctx, gbz, q)
        ch1 = np.zeros((lq, 2), dtype=np.uint64)
        ctx.check(gbz.lib.gbz_whir_update_betas(ctx.h, b1.p, b.shape[0], q1.p, lq, 1 << logN, r.ctypes.data,
                                                ch1.ctypes.data, gbz.MEM_DEVICE))
        ctx.synchronize()
        # no-allocation entry point on the default stream
        b2, q2 = DevBuf(ctx, gbz, b), DevBuf(ctx, gbz, q)
        ch2 = DevBuf(ctx, gbz, np.zeros((lq, 2), dtype=np.uint64))
        st = gbz.lib.gbz_whir_update_betas_noalloc(b2.p, b.shape[0], q2.p, lq, 1 << logN, r.ctypes.data, ch2.p, None)
        assert st == gbz.OK
        assert rt.cudaDeviceSynchronize() == 0
        assert np.array_equal(b2.read(b), b1.read(b))
        assert np.array_equal(ch2.read(ch1), ch1)
        for buf in (b1, q1, b2, q2, ch2):
            buf.free()


def test_empty_beta_vector_writes_the_weights_in_both_entry_points(ctx, gbz):
    """nb = 0: nothing to update, the l combination weights still written,
    the same by both entry points."""
    rng = np.random.default_rng(7)
    rt = _cudart()
    q = rng.integers(0, 1 << 12, size=20).astype(np.int32)
    r = rand_fe(rng, 1)[0].copy()
    b = np.zeros((1, 2), dtype=np.uint64)
    b1, q1 = DevBuf(ctx, gbz, b), DevBuf(ctx, gbz, q)
    ch1 = np.zeros((20, 2), dtype=np.uint64)
    ctx.check(gbz.lib.gbz_whir_update_betas(ctx.h, b1.p, 0, q1.p, 20, 1 << 12, r.ctypes.data, ch1.ctypes.data,
                                            gbz.MEM_DEVICE))
    ch2 = DevBuf(ctx, gbz, np.zeros((20, 2), dtype=np.uint64))
    assert gbz.lib.gbz_whir_update_betas_noalloc(b1.p, 0, q1.p, 20, 1 << 12, r.ctypes.data, ch2.p, None) == gbz.OK
    assert rt.cudaDeviceSynchronize() == 0
    assert np.array_equal(ch2.read(ch1), ch1)
    assert ch1[1].tolist() != [0, 0]
    for buf in (b1, q1, ch2):
        buf.free()


def test_noalloc_rejects_more_queries_than_its_scratch_holds(ctx, gbz):
    b = np.zeros((16, 2), dtype=np.uint64)
    q = np.zeros(257, dtype=np.int32)
    db, dq = DevBuf(ctx, gbz, b), DevBuf(ctx, gbz, q)
    r = np.array([3, 4], dtype=np.uint64)
    try:
        assert gbz.lib.gbz_whir_update_betas_noalloc(db.p, 16, dq.p, 257, 1 << 10, r.ctypes.data, None,
                                                     None) == gbz.EINVAL
        assert gbz.lib.gbz_whir_update_betas_noalloc(db.p, 16, dq.p, 4, 1000, r.ctypes.data, None,
                                                     None) == gbz.EINVAL
    finally:
        db.free()
        dq.free()
