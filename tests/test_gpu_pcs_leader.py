"""The whole of PCS_open_new on one device (gbz_pcs_open_full): the parties'
rounds of gbz_pcs_open, then the leader's tail, against the reference's own
coPCS test run with N = 4, 8 and 16 MPI ranks.

The tail draws only from rank 0's glibc generator.  The fixtures
(tests/golden/parties_*.json, "leader", written by tests/golden/make_golden.py
through oracle/ref's pigeon_mpi) hold what rank 0 computed after the parties'
rounds, and where its generator stood when the tail began.  Compared here:
- per delegate check after the first:
  - the root of the WHIR commitment to the gathered segments
  - the extension query draws
  - the claims of prove_multi_folding and prove_extension
  - the evaluations their checks compute
  - the extended segments at the queries
- aggregate_claims: K and its challenges
- the openings of aggregate_commitments
- per iteration of _Whir_Open:
  - its commitment root
  - its query draws
  - the roots of the replies it hashes
- _Whir_Open's final claim
- delegate_beta_eval: its claim and the evaluations of its check
- the messages the reference printed, against the flags
- the generator's final state.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest

pytestmark = pytest.mark.gpu

CASES = ["parties_N4_M14.json", "parties_N16_M16.json", "parties_N8_M19.json", "parties_N16_M24.json"]
(D_ROOT, D_QUERIES, D_POLYS, D_FINAL, D_CLAIM, D_OPEN, D_EXT, UNPACKED, WHIR_CLAIM, RC, BETA_Y,
 L_EVALS) = range(46, 58)
W_CHAL, W_ROOT, W_QUERIES, W_REPLIES, FINAL_EVAL = 8, 9, 10, 11, 18
AGGR_CH, AGGR_K, AGGR_Q = 20, 21, 22


def load(name):
    with open(os.path.join(conftest.GOLDEN, name)) as f:
        return json.load(f)


def point(gbz, n):
    fs = np.zeros(2, dtype=np.uint64)
    r = []
    for _ in range(n):
        fs = gbz.hash_to_field(fs, np.zeros((1, 2), dtype=np.uint64))
        r.append(fs.copy())
    return np.array(r, dtype=np.uint64), fs


def gen(gbz, state, calls=0):
    """A gbz.Prng in the oracle generator state `state`, `calls` random()
    calls further on."""
    import ctypes

    import gbz_oracle

    o = gbz_oracle.Prng.from_state(state)
    o.skip(calls)
    g = gbz.Prng(1)
    ctypes.memmove(ctypes.addressof(g), o.state(), ctypes.sizeof(g))
    return g


@pytest.fixture(scope="module", params=CASES)
def run(request, gbz, oracle, ctx):
    case = load(request.param)
    lead = case["leader"]
    N, M, rates = case["N"], 1 << case["logM"], case["rates"]
    deg, q, rnd = gbz.pcs_schedule(N, M, rates)
    # rank 0's generator after dealing the shares: nothing else draws from
    # it before the leader's tail (the tail's first draws check this)
    shares, random, g0 = oracle.copcs_party_shares(N, M, rnd * N // 4, state=True)
    com, _, _ = gbz.pcs_commit(ctx, N, M, rates, shares, random)
    r, fs = point(gbz, case["point_len"])
    K = np.frombuffer(bytes.fromhex(case["K"]), dtype=np.uint64)
    g = gen(gbz, g0)
    tr, _, flags = com.open_full(r, K, fs, g)
    recs = gbz.parse_transcript(tr)
    com.free()
    yield case, lead, deg, tr, recs, flags, (g, g0)


def by_tag(recs, tag):
    return [p for t, c, p in recs if t == tag]


def tail(recs):
    """The records after the parties' ones (from the first D_ROOT)."""
    i = next(k for k, (t, _, _) in enumerate(recs) if t == D_ROOT)
    return recs[i:]


def fes(p):
    return [p[16 * i:16 * i + 16].hex() for i in range(len(p) // 16)]


def test_parties_part_unchanged(run):
    case, _, _, tr, _, _, _ = run
    n = case["gpu_transcript_bytes"]
    assert hashlib.sha256(tr[:n]).hexdigest() == case["gpu_transcript_sha256"]


def test_delegation_rounds(run):
    case, lead, deg, _, recs, _, _ = run
    t = tail(recs)
    roots, qs, claims = by_tag(t, D_ROOT), by_tag(t, D_QUERIES), by_tag(t, D_CLAIM)
    opens, exts, fins = by_tag(t, D_OPEN), by_tag(t, D_EXT), by_tag(t, D_FINAL)
    assert len(roots) == len(lead["rounds"])
    for k, rd in enumerate(lead["rounds"]):
        i = k + 1                                   # the parties' round that delegates
        C0 = deg[i + 1] * case["rates"][i + 1][1]   # C[0].size(): the previous concatenated code's rows
        assert roots[k].hex() == rd["root"], k
        assert np.frombuffer(qs[k], dtype=np.uint32).tolist() == [x % C0 for x in rd["queries2"]], k
        pmf = fes(bytes.fromhex(rd["pmf"]))
        got = fes(claims[k])
        assert got[:len(pmf)] == pmf, k
        assert all(x == "00" * 16 for x in got[len(pmf):]), k
        assert exts[k].hex() == rd["pex"], k
        assert hashlib.sha256(opens[k]).hexdigest() == rd["pexo_sha256"], k
        # the evaluations of checks 4 and 7: the reduced matrix at the quadratic
        # sumcheck's point, prove_fft's phi vector at its point
        quad, pf = fins[4 * k + 1], fins[4 * k + 3]
        assert rd["check_evals"] == [fes(quad)[1], fes(pf)[0]], k


def test_aggregation_and_whir_opening(run, oracle):
    _, lead, _, _, recs, _, _ = run
    t = tail(recs)
    assert by_tag(t, AGGR_K)[0].hex() == lead["aggr_K"]
    assert by_tag(t, AGGR_CH)[0].hex() == lead["aggr_challenges"]
    # the aggregated codeword: the segments' WHIR commitments at rate 4 over
    # max_delegation = 2^(point length) entries
    Lw = 4 << (len(bytes.fromhex(lead["whir_claim"])) // 16 - 1)
    aq = np.frombuffer(by_tag(t, AGGR_Q)[0], dtype=np.uint32).tolist()
    assert aq == [x % (Lw // 4) for x in lead["aggr_queries"]]
    roots, wq, reps = by_tag(t, W_ROOT), by_tag(t, W_QUERIES), by_tag(t, W_REPLIES)
    its = lead["whir_iterations"]
    assert len(roots) == len(its)
    L_old = Lw
    for k, it in enumerate(its):
        assert roots[k].hex() == it["root"], k
        # whir_k = 8: the queries are rand() % (codeword / 8) of the codeword they open
        q = np.frombuffer(wq[k], dtype=np.uint32).tolist()
        assert q == [x % (L_old // 8) for x in it["queries"]], k
        rep = np.frombuffer(reps[k], dtype=np.uint64).reshape(-1, 8, 2)
        rr = b"".join(oracle.merkle_commit(rep[j])[-1].tobytes() for j in range(rep.shape[0]))
        assert hashlib.sha256(rr).hexdigest() == it["reply_roots_sha256"], k
        L_old = it["commit"]
    wc = by_tag(t, WHIR_CLAIM)[0]
    assert wc.hex() == lead["whir_claim"]
    assert lead["whir_evals"] == [by_tag(t, FINAL_EVAL)[-1].hex(), fes(wc)[0]]


def test_beta_delegation(run):
    _, lead, _, _, recs, _, _ = run
    t = tail(recs)
    assert by_tag(t, BETA_Y)[0].hex() == lead["beta_eval_y"]
    assert fes(by_tag(t, L_EVALS)[0]) == lead["beta_eval_evals"]


def test_flags_match_the_reference_messages(run):
    case, _, _, _, _, flags, _ = run
    out = "\n".join(case["stdout"])
    expect = 0
    if "Error in sumcheck round" in out:
        expect |= 1
    if "Error in final verification step 1" in out:
        expect |= 8
    if "Error in verification step 3" in out:
        expect |= 32
    assert flags == expect


def test_generator_ends_where_the_reference_does(run, gbz):
    """The tail made as many random() calls as rank 0 did after the dealing."""
    _, lead, _, _, _, _, (g, g0) = run
    assert bytes(g) == bytes(gen(gbz, g0, lead["prng_calls"]))
