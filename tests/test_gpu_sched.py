"""Many-proof scheduler: batched and served proofs are bit-identical to the
same proofs run alone (and to the reference's own transcripts where a
golden digest exists), whatever the mix, the slot count or graph replay.
"""
import hashlib

import numpy as np
import pytest

from conftest import splitmix_base

pytestmark = pytest.mark.gpu


def _mix(oracle, shapes, seed0=7000):
    ws, ln, rt, sd = [], [], [], []
    for k, (logn, rate) in enumerate(shapes):
        ws.append(oracle.witness(seed0 + k, 1 << logn))
        ln.append(logn)
        rt.append(rate)
        sd.append(1 + (k * 7919) % 1000)
    return ws, ln, rt, sd


SHAPES = [(12, 4), (8, 2), (14, 4), (10, 2), (12, 4), (9, 8), (16, 4), (13, 2), (11, 4), (15, 2), (12, 4), (7, 4)]


@pytest.fixture(scope="module")
def alone(ctx, oracle):
    ws, ln, rt, sd = _mix(oracle, SHAPES)
    ref = [ctx.prove(w, l, r, s).tobytes() for w, l, r, s in zip(ws, ln, rt, sd)]
    return ws, ln, rt, sd, ref


@pytest.mark.parametrize("lanes,graphs", [(1, False), (1, True), (4, True), (8, False), (8, True), (16, True)])
def test_batch_equals_alone(ctx, alone, lanes, graphs):
    ws, ln, rt, sd, ref = alone
    out, lat, mk = ctx.prove_batch(ws, ln, rt, sd, lanes=lanes, graphs=graphs)
    for k in range(len(ws)):
        assert out[k].tobytes() == ref[k], "proof %d differs in the batch" % k
    assert np.all(lat > 0) and mk >= lat.max() - 1e-9


@pytest.mark.parametrize("grouped", [True, False])
def test_batch_groups_of_one_shape(ctx, oracle, grouped):
    """Many proofs of a few shapes: grouped, every launch covers a whole
    shape group (batched plans); the transcripts are the ones each proof
    gives alone, with and without graph replay.  The shapes reach the sparse
    update_betas transform (2^16 at rate 4, 2^17 at rate 2), the one-CTA
    sumcheck tail (2^10) and the first fold without the eq table (2^3)."""
    shapes = [(12, 4)] * 9 + [(16, 4)] * 5 + [(17, 2)] * 3 + [(10, 8)] * 2 + [(3, 2)] * 2
    ws, ln, rt, sd = _mix(oracle, shapes, seed0=9100)
    ref = [ctx.prove(w, l, r, s).tobytes() for w, l, r, s in zip(ws, ln, rt, sd)]
    ctx.set_grouping(grouped)
    try:
        for graphs in (True, False):
            out, lat, mk = ctx.prove_batch(ws, ln, rt, sd, lanes=4, graphs=graphs)
            for k in range(len(ws)):
                assert out[k].tobytes() == ref[k], "proof %d (2^%d, rate %d) differs" % (k, ln[k], rt[k])
            assert np.all(lat > 0) and mk >= lat.max() - 1e-9
    finally:
        ctx.set_grouping(True)


def test_batch_repeat_uses_cached_graphs(ctx, alone):
    ws, ln, rt, sd, ref = alone
    for _ in range(3):
        out, _, _ = ctx.prove_batch(ws, ln, rt, sd, lanes=4)
        assert [o.tobytes() for o in out] == ref


def test_batch_pinned_host_buffers(ctx, gbz, alone):
    ws, ln, rt, sd, ref = alone
    pins = [gbz.PinnedArray(w.shape, np.uint64) for w in ws]
    for p, w in zip(pins, ws):
        p.array[...] = w
    outs = [gbz.PinnedArray((gbz.transcript_bytes(l, r),), np.uint8) for l, r in zip(ln, rt)]
    got, _, _ = ctx.prove_batch([p.array for p in pins], ln, rt, sd, lanes=6, out=[o.array for o in outs])
    assert [g.tobytes() for g in got] == ref


def test_batch_device_buffers(ctx, gbz, alone):
    torch = pytest.importorskip("torch")
    ws, ln, rt, sd, ref = alone
    dw = [torch.from_numpy(w.view(np.int64)).cuda() for w in ws]
    dt = [torch.zeros(gbz.transcript_bytes(l, r), dtype=torch.uint8, device="cuda") for l, r in zip(ln, rt)]
    for graphs in (True, False):
        for t in dt:
            t.zero_()
        ctx.prove_batch(dw, ln, rt, sd, lanes=4, graphs=graphs, out=dt)
        torch.cuda.synchronize()
        assert [t.cpu().numpy().tobytes() for t in dt] == ref


def test_batch_reference_digest_in_mix(ctx, golden, oracle):
    """The reference's 2^18 rate-1/4 transcript, proved inside a mixed batch."""
    e = next(x for x in golden["prove"] if x["logn"] == 18 and x["rate"] == 4)
    w = splitmix_base(e["seed"], 1 << 18)
    ws, ln, rt, sd = _mix(oracle, [(12, 4), (16, 2), (14, 4), (10, 4)], seed0=9000)
    ws.insert(2, w)
    ln.insert(2, 18)
    rt.insert(2, 4)
    sd.insert(2, e["prng_seed"])
    out, _, _ = ctx.prove_batch(ws, ln, rt, sd, lanes=3)
    t = out[2].tobytes()
    assert len(t) == e["bytes"]
    assert hashlib.sha256(t).hexdigest() == e["sha256"]


def test_serve_equals_alone(ctx, alone):
    ws, ln, rt, sd, ref = alone
    rng = np.random.default_rng(3)
    arrivals = np.cumsum(rng.exponential(1 / 400.0, size=len(ws)))
    out, lat, mk = ctx.serve(arrivals, ws, ln, rt, sd, lanes=4, depth=2)
    for k in range(len(ws)):
        assert out[k].tobytes() == ref[k], "served proof %d differs" % k
    assert np.all(lat > 0)
    assert mk >= arrivals.max()


def test_serve_burst_and_depth_one(ctx, alone):
    """All requests at t = 0 with one proof per slot in flight."""
    ws, ln, rt, sd, ref = alone
    out, lat, _ = ctx.serve(np.zeros(len(ws)), ws, ln, rt, sd, lanes=3, depth=1)
    assert [o.tobytes() for o in out] == ref
    assert np.all(lat > 0)


def test_serve_admission_refuses_what_cannot_fit(ctx, gbz, alone):
    """A shape with no cached plan is admitted only when its plan plus the
    reserve fits in free device memory; cached plans are evicted first."""
    ws, ln, rt, sd, ref = alone
    ctx.sched_release()
    with pytest.raises(gbz.GbzError) as ei:
        ctx.serve([0.0], ws[:1], ln[:1], rt[:1], sd[:1], lanes=1, reserve=1 << 50)
    assert ei.value.status == gbz.ENOMEM
    # the context stays usable
    out, _, _ = ctx.serve([0.0], ws[:1], ln[:1], rt[:1], sd[:1], lanes=1)
    assert out[0].tobytes() == ref[0]


def test_sched_invalid_arguments(ctx, gbz, oracle):
    w = oracle.witness(1, 1 << 8)
    with pytest.raises(gbz.GbzError) as ei:
        ctx.prove_batch([w], [8], [3], [1])
    assert ei.value.status == gbz.EINVAL
    with pytest.raises(gbz.GbzError) as ei:
        ctx.prove_batch([w], [8], [2], [1], out=[np.zeros(16, np.uint8)])
    assert ei.value.status == gbz.ESMALL
    with pytest.raises(gbz.GbzError):
        ctx.serve([-1.0], [w], [8], [2], [1])
    out, lat, mk = ctx.prove_batch([], [], [], [])
    assert out == [] and mk == 0.0


def test_sched_release(ctx, alone):
    ws, ln, rt, sd, ref = alone
    ctx.prove_batch(ws[:3], ln[:3], rt[:3], sd[:3], lanes=2)
    assert ctx.sched_release() > 0
    assert ctx.sched_release() == 0
    out, _, _ = ctx.prove_batch(ws[:3], ln[:3], rt[:3], sd[:3], lanes=2)
    assert [o.tobytes() for o in out] == ref[:3]
