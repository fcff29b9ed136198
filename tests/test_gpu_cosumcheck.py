"""quadratic_coSumcheck / cubic_coSumcheck of N parties on one device
(gbz_cosumcheck) against the reference's own functions run with N = 4, 8
and 16 ranks (tests/golden/cosumcheck.json, written through oracle/ref's
pigeon_cosc by tests/golden/make_golden.py).

The inputs are regenerated here exactly as the reference driver draws them
(oracle/ref/cosumcheck_mpi_driver.cpp); the whole transcript (every party's
round messages, the leader's aggregates, challenges, final shares and their
unpack), the claims and the check flags must equal the reference's.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest

pytestmark = pytest.mark.gpu
M64 = (1 << 64) - 1


def load():
    with open(os.path.join(conftest.GOLDEN, "cosumcheck.json")) as f:
        return json.load(f)


def driver_inputs(form, N, logn, degs, seed):
    """Rank p's draws of cosumcheck_mpi_driver.cpp: p1, p2, R[i] ... (p3),
    then r1, r2 from the stream shared by all ranks."""
    n = 1 << logn
    cubic = form == "cubic"
    step = 4 if cubic else 2
    P1, P2, P3, RR = [], [], [], []
    for p in range(N):
        s0 = (seed * 0x10001 + p * 0x9E3779B1 + 7) & M64
        count = 2 * n + sum(step * d for d in degs) + (n if cubic else 0)
        raw = conftest.splitmix_ext(s0, count)
        p1, p2 = raw[:n].copy(), raw[n:2 * n]
        off = 2 * n
        R = raw[off:off + sum(step * d for d in degs)]
        off += R.shape[0]
        if cubic:
            P3.append(raw[off:off + n])
            zb = int(np.prod(degs))
            for j in range(0, n // zb, 5):
                p1[j * zb:(j + 1) * zb] = 0
        P1.append(p1)
        P2.append(p2)
        RR.append(R)
    r1 = r2 = None
    if cubic:
        lk = (N // 4).bit_length() - 1
        g = conftest.splitmix_ext((seed * 0x7F4A7C15 + 3) & M64, logn + lk)
        r1, r2 = g[:logn], g[logn:]
    stack = lambda xs: np.ascontiguousarray(np.stack(xs)) if xs else None
    return stack(P1), stack(P2), stack(P3), stack(RR), r1, r2


@pytest.mark.parametrize("name", sorted(load()))
def test_cosumcheck_equals_reference(gbz, ctx, name):
    case = load()[name]
    form, N, logn, degs = case["form"], case["N"], case["logn"], case["degrees"]
    p1, p2, p3, R, r1, r2 = driver_inputs(form, N, logn, degs, case["seed"])
    cubic = form == "cubic"
    form_id = gbz.SC_CUBIC if cubic else gbz.SC_QUADRATIC
    K = np.frombuffer(bytes.fromhex(case["K"]), dtype=np.uint64)
    Kr = np.frombuffer(bytes.fromhex(case["K_r"]), dtype=np.uint64)
    claims, flags, tr, _ = gbz.cosumcheck(ctx, form_id, N, p1, p2, R, K, Kr, degs, p3=p3, r1=r1, r2=r2)
    assert len(tr) == case["transcript_bytes"]
    assert hashlib.sha256(tr).hexdigest() == case["transcript_sha256"]
    assert flags == case["flags"]
    # the leader's claims: (eval, [r_final, r_0, ...]) per row
    ref = bytes.fromhex(case["claims"])
    cnt = int(np.frombuffer(ref[:4], dtype=np.uint32)[0])
    assert cnt == len(claims)
    o = 4
    for ev, r in claims:
        assert ref[o:o + 16] == ev.tobytes()
        ln = int(np.frombuffer(ref[o + 16:o + 20], dtype=np.uint32)[0])
        assert ref[o + 20:o + 20 + 16 * ln] == r.tobytes()
        o += 20 + 16 * ln
