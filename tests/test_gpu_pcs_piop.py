"""PCS_open_new in the PIOP mode (isPIOP = true, coPCS.cpp:1310-1690, as
coPIOP_prove calls it, coPIOP.cpp:1741-1773) on one device
(gbz_pcs_open_piop), against the reference run unmodified with N = 8, 16 and 32
MPI ranks (tests/golden/pcspiop_*.json, written by tests/golden/make_golden.py
through oracle/ref's pigeon_dpcs pcs mode).

The inputs are the reference driver's: the coPCS test's dealing and
PCS_commit, then b1 = the Lagrange vector over 32 points, b2 = the tensor of
two Lagrange vectors over the row length (also passed as its factors), b3 =
the one over N/4 points, at four points of a SplitMix64 stream; K their F_ip
claim.  Compared:
- the parties' records: the whole transcript up to the leader's tail
- per delegation round: the WHIR root of the gathered segments, the
  extension query draws, the claims and the evaluations of the checks
- r_c
- delegate_lagrange_eval: its claim y and the evaluations of its checks
  (the rounds' Lagrange vectors, then the input's factors)
- the WHIR batch slots 2 and 3 the opening fills
- the flags against the reference's messages
- the generator's final state.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest
from test_gpu_pcs_leader import D_CLAIM, D_EXT, D_FINAL, D_OPEN, D_QUERIES, D_ROOT, L_EVALS, RC, BETA_Y, by_tag, \
    fes, gen, tail

pytestmark = pytest.mark.gpu

CASES = ["pcspiop_N8_M16.json", "pcspiop_N16_M16.json", "pcspiop_N16_M18.json", "pcspiop_N32_M17.json"]
LAG_EVALS = 69
AGGR_K, W_ROOT = 21, 9
M64 = (1 << 64) - 1


def load(name):
    with open(os.path.join(conftest.GOLDEN, name)) as f:
        return json.load(f)


def tensor(oracle, a, b):
    """out[k + j |a|] = b[j] a[k] (the reference's Lagrange_evals product)."""
    A = np.tile(a, (b.shape[0], 1))
    B = np.repeat(b, a.shape[0], axis=0)
    return oracle.field_ops(A, B)[2]


def inputs(oracle, N, Bs, seed):
    """The driver's input vectors (oracle/ref/dpcs_mpi_driver.cpp pcs mode)."""
    p = conftest.splitmix_ext((seed * 0x7F4A7C15 + 3) & M64, 4)
    lB = Bs.bit_length() - 1
    la, lb, lk = lB // 2, lB - lB // 2, (N // 4).bit_length() - 1
    b1 = oracle.lagrange_coeff(p[0], 5)
    La, Lb = oracle.lagrange_coeff(p[1], la), oracle.lagrange_coeff(p[2], lb)
    b3 = oracle.lagrange_coeff(p[3], lk)
    return b1, tensor(oracle, La, Lb), b3, [La, Lb]


@pytest.fixture(scope="module", params=CASES)
def run(request, gbz, oracle, ctx):
    case = load(request.param)
    N, M, rates = case["N"], 1 << case["logM"], case["rates"]
    deg, q, rnd = gbz.pcs_schedule(N, M, rates)
    shares, random, g0 = oracle.copcs_party_shares(N, M, rnd * N // 4, state=True)
    com, _, _ = gbz.pcs_commit(ctx, N, M, rates, shares, random)
    b1, b2, b3, lag = inputs(oracle, N, com.row_len, case["seed"])
    K_gpu = com.claim_piop(b1, b2, b3)
    K = np.frombuffer(bytes.fromhex(case["K"]), dtype=np.uint64)
    g = gen(gbz, g0)
    tr, _, flags, slots = com.open_piop(b1, b2, b3, lag, K, np.zeros(2, np.uint64), g)
    recs = gbz.parse_transcript(tr)
    com.free()
    yield case, deg, tr, recs, flags, slots, (g, g0, K_gpu)


def test_claim_equals_reference(run):
    """gbz_pcs_claim_piop: F_ip with the input vectors, as the reference's
    driver forms K for this opening."""
    case, _, _, _, _, _, (_, _, K_gpu) = run
    assert K_gpu.tobytes().hex() == case["K"]


def test_parties_part_equals_reference(run):
    case, _, tr, _, _, _, _ = run
    n = case["gpu_transcript_bytes"]
    assert hashlib.sha256(tr[:n]).hexdigest() == case["gpu_transcript_sha256"]


def test_delegation_rounds(run):
    case, deg, _, recs, _, _, _ = run
    lead = case["leader"]
    t = tail(recs)
    roots, qs, claims = by_tag(t, D_ROOT), by_tag(t, D_QUERIES), by_tag(t, D_CLAIM)
    exts, fins, opens = by_tag(t, D_EXT), by_tag(t, D_FINAL), by_tag(t, D_OPEN)
    assert len(roots) == len(lead["rounds"])
    for k, rd in enumerate(lead["rounds"]):
        i = k + 1
        C0 = deg[i + 1] * case["rates"][i + 1][1]
        assert roots[k].hex() == rd["root"], k
        assert np.frombuffer(qs[k], dtype=np.uint32).tolist() == [x % C0 for x in rd["queries2"]], k
        pmf = fes(bytes.fromhex(rd["pmf"]))
        got = fes(claims[k])
        assert got[:len(pmf)] == pmf, k
        assert all(x == "00" * 16 for x in got[len(pmf):]), k
        assert exts[k].hex() == rd["pex"], k
        assert hashlib.sha256(opens[k]).hexdigest() == rd["pexo_sha256"], k
        quad, pf = fins[4 * k + 1], fins[4 * k + 3]
        assert rd["check_evals"] == [fes(quad)[1], fes(pf)[0]], k


def test_no_aggregation_or_whir_opening(run):
    _, _, _, recs, _, _, _ = run
    t = tail(recs)
    assert not by_tag(t, AGGR_K) and not by_tag(t, W_ROOT)


def test_rc(run):
    case, _, _, recs, _, _, _ = run
    assert fes(by_tag(tail(recs), RC)[0])[0] == case["leader"]["r_c"]


def test_lagrange_delegation(run):
    case, _, _, recs, _, _, _ = run
    lead = case["leader"]
    t = tail(recs)
    assert by_tag(t, BETA_Y)[0].hex() == lead["lag_y"]
    assert fes(by_tag(t, L_EVALS)[0]) + fes(by_tag(t, LAG_EVALS)[0]) == lead["lag_evals"]


def test_whir_slots(run):
    case, _, _, _, _, slots, _ = run
    for c, ref in enumerate(case["whir_slots"]):
        got = slots[c]
        for key in ("arr", "codeword", "betas"):
            n = ref[key + "_len"]
            v = got[key]
            assert hashlib.sha256(v[:n].tobytes()).hexdigest() == ref[key + "_sha256"], (c, key)
            assert not np.any(v[n:]), (c, key)
        assert got["claim"].tobytes().hex() == ref["claim"], c
        assert got["root"].tobytes().hex() == ref["root"], c


def test_flags_match_the_reference_messages(run):
    case, _, _, _, flags, _, _ = run
    out = "\n".join(case["stdout"])
    expect = 0
    if "Error in sumcheck round" in out:
        expect |= 1
    if "Error in final verification step 1" in out:
        expect |= 8
    if "Error in delegating betas 3" in out:
        expect |= 512
    assert flags == expect


def test_generator_ends_where_the_reference_does(run, gbz):
    case, _, _, _, _, _, (g, g0, _) = run
    assert bytes(g) == bytes(gen(gbz, g0, case["leader"]["prng_calls"]))


def test_inconsistent_factors_are_rejected(gbz, oracle, ctx):
    """Lagrange factors whose lengths do not multiply to the row length."""
    case = load(CASES[0])
    N, M, rates = case["N"], 1 << case["logM"], case["rates"]
    deg, q, rnd = gbz.pcs_schedule(N, M, rates)
    shares, random = oracle.copcs_party_shares(N, M, rnd * N // 4)
    com, _, _ = gbz.pcs_commit(ctx, N, M, rates, shares, random)
    b1, b2, b3, lag = inputs(oracle, N, com.row_len, case["seed"])
    with pytest.raises(gbz.GbzError):
        com.open_piop(b1, b2, b3, lag[:1], np.zeros(2, np.uint64), np.zeros(2, np.uint64), gbz.Prng(1))
    com.free()
