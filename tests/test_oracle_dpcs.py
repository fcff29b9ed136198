"""The oracle's restatement of the distributed PCS commitments
(oracle/gbz_dpcs_oracle.py) against the reference's Batch_dCommit and
dCommit run with 8, 16 and 32 ranks (tests/golden/dpcs.json): every rank's
codeword rows, commit data and tree levels by SHA-256, its root, and rank
0's leader root."""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest
import dpcs_cases


def cases():
    with open(os.path.join(conftest.GOLDEN, "dpcs.json")) as f:
        d = json.load(f)
    return [d[k] for k in sorted(d)]


def sha(b):
    return hashlib.sha256(np.ascontiguousarray(b).tobytes()).hexdigest()


@pytest.mark.parametrize("case", cases(), ids=lambda c: "%s_N%d_A%d" % (c["mode"], c["N"], c["logA"]))
def test_dpcs_oracle_matches_reference(case, oracle):
    import gbz_dpcs_oracle as do
    import gbz_oracle as orc
    arr, arr2 = dpcs_cases.driver_arrays(case)
    batch = case["mode"] == "batch"
    cw, lv, roots = do.commit(arr, case["batch"] if batch else 1, case["rate"],
                              None if batch else dpcs_cases.column_height(case["N"]))
    for p, rk in enumerate(case["ranks"]):
        assert sha(cw[p]) == rk["codewords_sha256"], p
        assert lv[p].shape[0] == rk["levels"] and sha(lv[p]) == rk["levels_sha256"], p
        assert roots[p].tobytes().hex() == rk["root"], p
        if batch:
            assert sha(arr2[p]) == rk["commit_data_sha256"], p
    # the leader's tree over {party 0's root, 0, ...}: its root is log2 N self-hashes
    h = roots[0].reshape(1, 32)
    for _ in range(case["N"].bit_length() - 1):
        h = orc.blake3_64(np.concatenate([h, h], axis=1))
    assert h[0].tobytes().hex() == case["ranks"][0]["leader_root"]
