"""The distributed PCS commitments of N parties on one device
(gbz_dpcs_batch_commit, gbz_dpcs_commit) against the reference's
Batch_dCommit and dCommit run with 8, 16 and 32 ranks
(tests/golden/dpcs.json): every party's codeword rows, commit data and tree
levels by SHA-256, its root, and the leader's root."""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest
import dpcs_cases

pytestmark = pytest.mark.gpu


def cases():
    with open(os.path.join(conftest.GOLDEN, "dpcs.json")) as f:
        d = json.load(f)
    return [d[k] for k in sorted(d) if d[k]["mode"] != "open"]


def sha(b):
    return hashlib.sha256(np.ascontiguousarray(b).tobytes()).hexdigest()


@pytest.mark.parametrize("case", cases(), ids=lambda c: "%s_N%d_A%d" % (c["mode"], c["N"], c["logA"]))
def test_dpcs_matches_reference(case, gbz, ctx):
    arr, arr2 = dpcs_cases.driver_arrays(case)
    if case["mode"] == "batch":
        cd, cw, lv, roots, lead = gbz.dpcs_batch_commit(ctx, arr, arr2, case["rate"], case["batch"])
    else:
        cw, lv, roots, lead = gbz.dpcs_commit(ctx, arr, case["rate"])
        cd = None
    for p, rk in enumerate(case["ranks"]):
        assert sha(cw[p]) == rk["codewords_sha256"], p
        assert lv[p].shape[0] == rk["levels"] and sha(lv[p]) == rk["levels_sha256"], p
        assert roots[p].tobytes().hex() == rk["root"], p
        if cd is not None:
            assert sha(cd[p]) == rk["commit_data_sha256"], p
    assert lead.tobytes().hex() == case["ranks"][0]["leader_root"]


def test_dpcs_rejects_bad_shapes(gbz, ctx):
    arr = np.zeros((4, 1024, 2), dtype=np.uint64)
    with pytest.raises(gbz.GbzError):
        gbz.dpcs_commit(ctx, arr, 4)                      # N = 4: below the supported parties
    arr = np.zeros((8, 1024, 2), dtype=np.uint64)
    with pytest.raises(gbz.GbzError):
        gbz.dpcs_batch_commit(ctx, arr, arr, 4, 2)       # batch below 4


def open_cases():
    with open(os.path.join(conftest.GOLDEN, "dpcs.json")) as f:
        d = json.load(f)
    return [d[k] for k in sorted(d) if d[k]["mode"] == "open"]


@pytest.mark.parametrize("case", open_cases(), ids=lambda c: "P%d_N%d_A%d" % (c["P"], c["N"], c["logA"]))
def test_dpcs_open_matches_reference(case, gbz, oracle, ctx):
    """The distributed opening (gbz_dpcs_open) on the commitments
    gbz_dpcs_batch_commit makes, against the reference's PIOP_dOpen_batch_new
    run with N ranks: every draw, the eval claims, the round messages, every
    party's commitment roots and query draws, the leader's roots, the
    gathered data, betas and claim, and the leader's WHIR commitment."""
    import struct
    import gbz_dpcs_oracle as do
    import gbz_oracle as orc
    P, N, rate, nb = case["P"], case["N"], case["rate"], case["batch"]
    _, _, arrs_all, r, y = dpcs_cases.open_inputs(case, orc)
    A = 1 << case["logA"]
    cds, cws = [], []
    for l in range(P):
        arr2 = np.zeros_like(arrs_all[l])
        if l == 0:
            arr2 = np.stack([conftest.splitmix_ext((case["seed"] * 0x10001 + p * 0x9E3779B1 + 11) & dpcs_cases.M64,
                                                   2 * A)[A:] for p in range(N)])
        cd, cw, _, _, _ = gbz.dpcs_batch_commit(ctx, arrs_all[l], arr2, rate, nb)
        cds.append(cd.reshape(N, nb, A // nb, 2))
        cws.append(cw)
    arr, bet, K, wc, root, flags, tr, fs = gbz.dpcs_open(ctx, np.stack(cds), np.stack(cws), np.stack(r), np.stack(y),
                                                        rate, rate)
    assert flags == 0
    recs = gbz.parse_transcript(tr)
    tag = lambda t: [p for k, c, p in recs if k == t]
    assert tag(61)[0].hex() == case["eval_claims"]
    dr = tag(62)[0]
    draws = [dr[16 * i:16 * i + 16].hex() for i in range(4)] + [c.hex() for c in tag(66)]
    assert draws == case["draws"]
    assert [p.hex() for p in tag(65)] == case["round_polys"]
    roots = tag(63)
    assert [x[32 * N:].hex() for x in roots] == case["leader_roots"]
    l = dpcs_cases.query_count(rate)
    degs = do.fold_degrees(N)
    L = A // nb * rate
    Ms = [L] + [L // (degs[0]) // degs[0]]
    for p, rk in enumerate(case["ranks"]):
        assert [x[32 * p:32 * p + 32].hex() for x in roots] == rk["roots"], p
        got = []
        for t, qb in enumerate(tag(64)):
            q = np.frombuffer(qb, dtype=np.uint32).reshape(-1, 2)
            w = [l, N, Ms[t], p] + [int(x) for pr in q if pr[0] == p for x in pr]
            got.append(hashlib.sha256(struct.pack("<%dI" % len(w), *w)).hexdigest())
        assert got == rk["queries"], p
    assert sha(arr) == case["whir_arr_sha256"] and sha(bet) == case["whir_betas_sha256"]
    assert K.tobytes().hex() == case["whir_claim"]
    assert sha(wc) == case["whir_codeword_sha256"] and root.tobytes().hex() == case["whir_root"]
    assert tag(68)[0].hex() == case["whir_root"]
