"""The N-party restatement (oracle/gbz_pcs_oracle.py) against the reference's
own coPCS test run with N = 4 and 16 ranks (tests/golden/parties_*.json,
written through oracle/ref's pigeon_mpi by tests/golden/make_golden.py).

What is compared, rank by rank: the packed-Shamir shares rank 0 deals from
glibc's default state, the distributed_MT roots, the opening claim K, every
Fiat-Shamir challenge of the opening, every party's local round message and
the leader's aggregate, every rank's queries, the delegate_checks answers
and segments, the batch / concatenated / tensor-code roots (including the
stale root that commit_tensorcode reports) and the final data each party
sends the leader.
"""
import hashlib
import json
import math
import os

import numpy as np
import pytest

import conftest

CASES = ["parties_N4_M14.json", "parties_N16_M16.json"]


def load(name):
    with open(os.path.join(conftest.GOLDEN, name)) as f:
        return json.load(f)


def fe_hex(values):
    return np.array(values, dtype=np.uint64).reshape(-1, 2).tobytes().hex()


@pytest.fixture(scope="module")
def pcs(oracle):
    import gbz_pcs_oracle

    return gbz_pcs_oracle


def run_case(oracle, pcs, case):
    N, M = case["N"], 1 << case["logM"]
    sched = pcs.schedule(N, M, case["rates"])
    shares, random = oracle.copcs_party_shares(N, M, sched["randomness"] * N // 4)
    parties = pcs.commit(sched, shares, random)
    chain = pcs.Chain()
    r = [chain.h2f([(0, 0)]) for _ in range(case["point_len"])]
    K = pcs.f_ip(parties, sched, r)
    out = pcs.open_parties(sched, parties, r, K, fs=chain.s)
    return sched, shares, random, parties, K, out


@pytest.mark.parametrize("name", CASES)
def test_schedule_matches_reference_printout(pcs, name):
    case = load(name)
    sched = pcs.schedule(case["N"], 1 << case["logM"], case["rates"])
    out = "\n".join(case["stdout"])
    assert "Degrees: " + "".join("%d, " % d for d in sched["degrees"]) in out
    assert "Queries: " + "".join("%d, " % q for q in sched["queries"]) in out


@pytest.mark.parametrize("name", CASES)
def test_parties_match_reference_ranks(oracle, pcs, name):
    case = load(name)
    N = case["N"]
    sched, shares, random, parties, K, out = run_case(oracle, pcs, case)
    for rk, e in enumerate(case["ranks"]):
        assert e["shares_sha256"] == [hashlib.sha256(shares[rk].tobytes()).hexdigest(),
                                      hashlib.sha256(random[rk].tobytes()).hexdigest()], rk
        assert e["base_root"] == parties[rk]["root"].hex(), rk
    assert case["K"] == fe_hex([K])
    # every challenge of the opening, in order: first round, then per round
    # the sumcheck challenge and phase 3's s
    seq = [out["challenges"][0]]
    for i in range(len(out["s"])):
        seq += [out["challenges"][1 + i], out["s"][i]]
    assert case["challenges"] == [fe_hex([c]) for c in seq]
    assert case["polys"] == [fe_hex(p) for p in out["polys"]]
    assert case["y"] == [fe_hex(y) for y in out["y"]]
    assert case["segments_sha256"] == [
        hashlib.sha256(bytes.fromhex(fe_hex([v for seg in segs for v in seg]))).hexdigest()
        for segs in out["segments"]]
    for rk, e in enumerate(case["ranks"]):
        assert e["party_polys"] == [fe_hex(pp[rk]) for pp in out["party_polys"]], rk
        mine = [[b for a, b in qd if a == rk] for _, qd in out["queries"]]
        assert e["queries"] == mine, rk
        roots = [out["roots"][k][1][rk].hex() for k in (1, 2, 3)]
        assert [x.split(":")[0] for x in e["commit_roots"]] == roots, rk
        # create_tree_blake roots: base tree, batch tree, and on the leader
        # the {root, 0, ...} trees; batch_commitments_new's base root is the
        # second one on every rank
        tr = [x.split(":")[0] for x in e["tree_roots"]]
        assert out["roots"][0][1][rk].hex() in tr, rk
        fin = out["final"][rk]
        assert e["final"] == [fin[0].tobytes().hex(), fin[1].tobytes().hex(), fin[2].tobytes().hex()], rk
    lead = [x.split(":") for x in case["ranks"][0]["tree_roots"]]
    leaders = [v for v, n in lead if int(n) == N]
    assert leaders[0] == parties[0]["leader"].hex()
    assert [r[2].hex() for r in out["roots"]] == leaders[1:1 + len(out["roots"])]


def test_tensorcode_root_is_the_previous_commitment_root(oracle, pcs):
    """commit_tensorcode reuses the previous tree's levels and MT_commit_Blake
    resizes only an empty levels vector (merkle_tree.cpp:205-208), so the
    reported root is the last concatenated commitment's root."""
    case = load(CASES[0])
    _, _, _, _, _, out = run_case(oracle, pcs, case)
    assert out["roots"][3][0] == "tensorcode" and out["roots"][3][1] == out["roots"][2][1]
