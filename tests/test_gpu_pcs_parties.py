"""The N-party collaborative PCS on one device (gbz_pcs_commit / gbz_pcs_open)
against the reference's own coPCS test run with N = 4, 8 and 16 MPI ranks
(tests/golden/parties_*.json: every rank's transcript, captured by
oracle/ref's pigeon_mpi; see tests/golden/make_golden.py).

The shares are the ones the reference's rank 0 deals (restated by the
oracle, which tests/test_oracle_parties.py pins to the fixtures' digests);
everything after them is computed on the GPU and compared byte for byte:
party roots and the leader's root of PCS_commit, then every party's round
message, the leader's aggregate, every Fiat-Shamir challenge, every rank's
queries, the delegate_checks answers and segments, every commitment root
(with commit_tensorcode's stale root) and the data each party finally sends.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest

pytestmark = pytest.mark.gpu

CASES = ["parties_N4_M14.json", "parties_N16_M16.json", "parties_N8_M19.json", "parties_N16_M24.json"]
T_ROOTS, T_LEADER, T_PP, T_POLY, T_CHAL, T_Q, T_Y, T_SEG, T_S, T_K, T_FINAL = range(32, 43)


def load(name):
    with open(os.path.join(conftest.GOLDEN, name)) as f:
        return json.load(f)


def point(gbz, n):
    """r = hash_to_field({0}) n times from prev_challenge = 0 (main.cpp:83-85)."""
    fs = np.zeros(2, dtype=np.uint64)
    r = []
    for _ in range(n):
        fs = gbz.hash_to_field(fs, np.zeros((1, 2), dtype=np.uint64))
        r.append(fs.copy())
    return np.array(r, dtype=np.uint64), fs


@pytest.fixture(scope="module", params=CASES)
def run(request, gbz, oracle, ctx):
    case = load(request.param)
    N, M, rates = case["N"], 1 << case["logM"], case["rates"]
    deg, q, rnd = gbz.pcs_schedule(N, M, rates)
    shares, random = oracle.copcs_party_shares(N, M, rnd * N // 4)
    com, roots, leader = gbz.pcs_commit(ctx, N, M, rates, shares, random)
    r, fs = point(gbz, case["point_len"])
    K = np.frombuffer(bytes.fromhex(case["K"]), dtype=np.uint64)
    tr, fs_after = com.open(r, K, fs)
    recs = gbz.parse_transcript(tr)
    yield case, (deg, q, rnd), shares, random, com, roots, leader, recs
    com.free()


def by_tag(recs, tag):
    return [p for t, c, p in recs if t == tag]


def test_whole_transcript_equals_reference(run, gbz):
    """The opening's whole transcript equals the one rebuilt from the
    reference ranks' records (tests/golden/make_golden.py,
    expected_open_transcript): one digest over every byte."""
    case, *_, recs = run
    blob = b"".join(np.array([t, c], dtype=np.uint32).tobytes() + p for t, c, p in recs)
    assert len(blob) == case["gpu_transcript_bytes"]
    assert hashlib.sha256(blob).hexdigest() == case["gpu_transcript_sha256"]


def test_schedule(run):
    case, (deg, q, rnd), *_ = run
    out = "\n".join(case["stdout"])
    assert "Degrees: " + "".join("%d, " % d for d in deg) in out
    assert "Queries: " + "".join("%d, " % x for x in q) in out


def test_commit_roots(run):
    case, _, _, _, com, roots, leader, _ = run
    for rk, e in enumerate(case["ranks"]):
        assert roots[rk].tobytes().hex() == e["base_root"], rk
    lead = [v for v, n in (x.split(":") for x in case["ranks"][0]["tree_roots"]) if int(n) == case["N"]]
    assert leader.tobytes().hex() == lead[0]


def test_commit_data_matches_oracle_restatement(run, oracle):
    """Commit_data rows and codewords of party 0 and the last party equal
    prepare_data + Encode of the restatement."""
    import gbz_pcs_oracle as po
    case, _, shares, random, com, *_ = run
    if case["logM"] > 16:
        pytest.skip("restatement too slow at this size (roots are compared with the reference instead)")
    sched = po.schedule(case["N"], 1 << case["logM"], case["rates"])
    for p in (0, case["N"] - 1):
        cd = po.prepare_data(shares[p], random[p], sched["queries"][0])
        rows, cws, _ = com.data(p)
        assert np.array_equal(rows, cd)
        assert np.array_equal(cws, oracle.encode_rows(cd, sched["rates"][0][0], 6))


def test_claim_equals_reference_F_ip(run, gbz):
    """gbz_pcs_claim gives the K that the reference's F_ip computed."""
    case, _, _, _, com, *_ = run
    r, _ = point(gbz, case["point_len"])
    assert com.claim(r).tobytes().hex() == case["K"]


def test_challenges_and_messages(run):
    case, *_, recs = run
    chal = [p.hex() for p in by_tag(recs, T_CHAL)]
    s = [p.hex() for p in by_tag(recs, T_S)]
    seq = [chal[0]]
    for i in range(len(s)):
        seq += [chal[1 + i], s[i]]
    assert seq == case["challenges"]
    assert [p.hex() for p in by_tag(recs, T_POLY)] == case["polys"]
    N = case["N"]
    pp = by_tag(recs, T_PP)
    for rk, e in enumerate(case["ranks"]):
        mine = []
        for p in pp:
            n = len(p) // N
            mine.append(p[rk * n:(rk + 1) * n])
        digest = len(e["party_polys"][0]) == 64 and len(mine[0]) != 32
        assert [hashlib.sha256(m).hexdigest() if digest else m.hex() for m in mine] == e["party_polys"], rk


def test_queries_answers_segments(run):
    case, *_, recs = run
    N = case["N"]
    qs = [np.frombuffer(p, dtype=np.uint32).reshape(-1, 2) for p in by_tag(recs, T_Q)]
    for rk, e in enumerate(case["ranks"]):
        mine = [[int(b) for a, b in q if a == rk] for q in qs]
        if e["queries"] and isinstance(e["queries"][0], str):
            mine = [hashlib.sha256(str(m).encode()).hexdigest() for m in mine]
        assert mine == e["queries"], rk
    assert [p.hex() for p in by_tag(recs, T_Y)] == case["y"]
    assert [hashlib.sha256(p).hexdigest() for p in by_tag(recs, T_SEG)] == case["segments_sha256"]


def test_roots_of_the_opening(run):
    case, *_, recs = run
    N = case["N"]
    rts = by_tag(recs, T_ROOTS)
    for rk, e in enumerate(case["ranks"]):
        tr = [x.split(":")[0] for x in e["tree_roots"]]
        assert rts[0][32 * rk:32 * rk + 32].hex() in tr, rk  # batch_commitments_new
        got = [r[32 * rk:32 * rk + 32].hex() for r in rts[1:]]
        assert got == [x.split(":")[0] for x in e["commit_roots"]], rk
    lead = [v for v, n in (x.split(":") for x in case["ranks"][0]["tree_roots"]) if int(n) == N]
    assert [p.hex() for p in by_tag(recs, T_LEADER)] == lead[1:1 + len(rts)]


def test_final_party_data(run):
    """send_pcs_data: every party's folded data, B and C' (full bytes for the
    small cases, SHA-256 for the large one)."""
    case, *_, recs = run
    N = case["N"]
    fin = by_tag(recs, T_FINAL)[0]
    per = len(fin) // N
    for rk, e in enumerate(case["ranks"]):
        blob = fin[rk * per:(rk + 1) * per]
        la, lb, lc = e["final_bytes"]
        assert la + lb + lc == per
        parts = [blob[:la], blob[la:la + lb], blob[la + lb:]]
        if len(e["final"][0]) == 64 and la != 32:
            got = [hashlib.sha256(x).hexdigest() for x in parts]
        else:
            got = [x.hex() for x in parts]
        assert got == e["final"], rk


def test_open_is_repeatable(run, gbz):
    """The commitment is read, not changed, by an opening."""
    case, _, _, _, com, _, _, recs = run
    r, fs = point(gbz, case["point_len"])
    K = np.frombuffer(bytes.fromhex(case["K"]), dtype=np.uint64)
    tr, _ = com.open(r, K, fs)
    assert gbz.parse_transcript(tr) == recs


def test_wrong_claim_is_rejected(run, gbz):
    case, _, _, _, com, *_ = run
    r, fs = point(gbz, case["point_len"])
    K = np.frombuffer(bytes.fromhex(case["K"]), dtype=np.uint64).copy()
    K[0] ^= 1
    with pytest.raises(gbz.GbzError) as e:
        com.open(r, K, fs)
    assert e.value.status == gbz.ECHECK
