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
    return [d[k] for k in sorted(d) if d[k]["mode"] != "open"]


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


def open_cases():
    with open(os.path.join(conftest.GOLDEN, "dpcs.json")) as f:
        d = json.load(f)
    return [d[k] for k in sorted(d) if d[k]["mode"] == "open"]


def gidx_sha(q, l, N, M, pos):
    import struct
    w = [l, N, M, pos] + [x for pr in q if pr[0] == pos for x in pr]
    return hashlib.sha256(struct.pack("<%dI" % len(w), *w)).hexdigest()


@pytest.mark.parametrize("case", open_cases(), ids=lambda c: "P%d_N%d_A%d" % (c["P"], c["N"], c["logA"]))
def test_dpcs_open_oracle_matches_reference(case, oracle):
    import gbz_dpcs_oracle as do
    import gbz_oracle as orc
    N, rate = case["N"], case["rate"]
    cd, cwg, _, r, y = dpcs_cases.open_inputs(case, orc)
    assert np.array(y).tobytes().hex() == case["y"]
    L = cwg[0].shape[1] // N
    l = dpcs_cases.query_count(rate)
    res = do.open_batch(cd, cwg, L, r, y, N, rate, l)
    assert res["flags"] == 0 and case["errors"] == []
    assert res["K"].tobytes().hex() == case["eval_claims"]
    draws = [res["a"][0], res["a"][1]] + [None, res["b1"]] + res["challenges"]
    assert [d.tobytes().hex() for i, d in enumerate(draws) if i != 2] == \
        [h for i, h in enumerate(case["draws"]) if i != 2]
    assert [p.tobytes().hex() for p in res["polys"]] == case["round_polys"]
    assert [x.tobytes().hex() for x in res["leader_roots"]] == case["leader_roots"]
    Ms = res["query_ranges"]
    for p, rk in enumerate(case["ranks"]):
        assert [res["roots"][t][p].tobytes().hex() for t in range(len(res["roots"]))] == rk["roots"], p
        got = [gidx_sha(res["queries"][t], l, N, Ms[t], p) for t in range(len(res["queries"]))]
        assert got == rk["queries"], p
    assert sha(res["codeword"]) == case["gathered_codeword_sha256"]
    # the leader's WHIR commitment of the gathered data (Whir_Commit_initial at the opening's rate)
    assert sha(res["arr"]) == case["whir_arr_sha256"] and sha(res["B"]) == case["whir_betas_sha256"]
    assert res["K_final"].tobytes().hex() == case["whir_claim"]
    wc = np.zeros((res["arr"].shape[0] * rate, 2), dtype=np.uint64)
    wc[:res["arr"].shape[0]] = res["arr"]
    wc = orc.fft(wc)
    assert sha(wc) == case["whir_codeword_sha256"]
    assert orc.merkle_commit(wc)[-1].tobytes().hex() == case["whir_root"]
