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
