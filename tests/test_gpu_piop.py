"""The R1CS front end's two sumcheck phases of N parties on one device
(gbz_piop_phase1 / gbz_piop_phase2, with gbz_r1cs_reduce and gbz_pcs_commit
on the way) against what the unmodified reference computed when its
`pigeon 1` ran with N = 8 and 16 ranks (tests/golden/piop_*.json).

The parties' inputs are the oracle's regeneration of rank 0's dealing
(pinned to every rank's digests by tests/test_oracle_piop.py).  Compared:
the phases' Fiat-Shamir draws, the vectors each phase hands its coSumcheck,
the coSumchecks' claims, every party's inner-product vectors, the reduced
R1CS rows, the second phase's a, b, c and the chain state after each phase.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest

pytestmark = pytest.mark.gpu

CASES = ["piop_N8_M16.json", "piop_N16_M16.json", "piop_N8_M18.json", "piop_N16_M20.json"]
RATES = [[4], [4], [4, 4], [4, 4]]


def load(name):
    with open(os.path.join(conftest.GOLDEN, name)) as f:
        return json.load(f)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint64).tobytes()).hexdigest()


def fes(hexes):
    b = b"".join(bytes.fromhex(h) for h in hexes)
    return np.frombuffer(b, dtype=np.uint64).reshape(-1, 2)


def ref_claims(blob, points):
    v = np.frombuffer(bytes.fromhex(blob), dtype=np.uint64).reshape(-1, 2)
    out, o = [], 0
    for n in points:
        out.append((v[o], v[o + 1:o + 1 + n]))
        o += 1 + n
    return out


def csr(parts):
    """The per-party CSR arrays of gbz_piop_oracle.r1cs_rows joined into one
    over all N x rows rows."""
    ptrs, cols, base = [np.zeros(1, dtype=np.int64)], [], 0
    for ptr, c in parts:
        ptrs.append(ptr[1:] + base)
        cols.append(c)
        base += c.shape[0]
    return np.concatenate(ptrs).astype(np.uint32), np.concatenate(cols).astype(np.uint32)


@pytest.fixture(scope="module", params=CASES)
def run(request, gbz, oracle, ctx):
    import gbz_piop_oracle as po
    case = load(request.param)
    N, M = case["N"], 1 << case["logM"]
    d = po.deal(N, M, case["generator"]["draws"][0][1], case["pcs_randomness"], case["mask_l"])
    masks = np.ascontiguousarray(d["R"][:, :12])
    # phase 1 from the chain state PCS_commit left
    fs0 = fes([case["fs0"]])[0]
    ph1 = gbz.piop_phase1(ctx, N, d["vL"], d["vR"], d["vO"], masks, d["R1"], d["degrees1"], fs0, vectors=True)
    # the witness of phase 2: the commitment's rows put back (coPIOP.cpp:1550-1563)
    com, _, _ = gbz.pcs_commit(ctx, N, d["W"].shape[1] * N // 4, RATES, d["W"], d["pcs_random"])
    rows_total = len(case["commit_rows"])
    w = []
    for p in range(N):
        rows, _, _ = com.data(p)
        lst = [rows[j] for j in range(rows.shape[0])]
        lst += [np.zeros((0, 2), dtype=np.uint64)] * (rows_total - len(lst))
        w.append(po.witness_layout(lst, com.row_len, case["mask_l"]))
    w = np.stack(w)
    cd = [com.data(p)[0] for p in range(N)]
    com.free()
    parts = po.r1cs_rows(d["circuit"], N)
    mats = [csr(parts[m]) for m in "ABC"]
    r1cs = gbz.R1cs(ctx, N, (1 << case["logn"]) // N, case["logm"], [m[0] for m in mats], [m[1] for m in mats])
    cl1 = ph1[0]
    point1 = cl1[0][1]
    evals1 = np.array([cl1[i][0] for i in range(3)])
    K = fes([case["K"]])[0]
    ph2 = gbz.piop_phase2(ctx, N, w, masks, r1cs, case["mask_l"], d["R2"], point1, evals1, d["degrees1"],
                          d["degrees2"], K, ph1[5], vectors=True)
    red = r1cs.reduce(point1[:-1], d["degrees1"])
    r1cs.free()
    yield case, d, ph1, ph2, red, cd


def test_phase1_draws_and_vectors(run, gbz):
    case, d, ph1, _, _, _ = run
    N = case["N"]
    recs = gbz.parse_transcript(ph1[4])
    ln, lk = d["vL"].shape[1].bit_length() - 1, (N // 4).bit_length() - 1
    assert recs[0][0] == 58
    assert [recs[0][2][16 * i:16 * i + 16].hex() for i in range(recs[0][1])] == case["draws"][:ln + lk + 1]
    vec = ph1[6]
    for p, rk in enumerate(case["ranks"]):
        h = rk["phase1_sha256"]
        assert (sha(vec[0][p]), sha(vec[1][p]), sha(vec[2][p])) == (h["p1"], h["p2"], h["p3"]), p
    # the leader's y and K_r: the coSumcheck's K = y r1[-1] and K_r
    y = np.frombuffer(recs[1][2], dtype=np.uint64).reshape(-1, 2)
    assert y[N + 1].tobytes().hex() == case["phase1"]["Kr"]


def test_phase1_claims_and_ip(run):
    case, _, ph1, _, _, _ = run
    ref = ref_claims(case["phase1"]["claims"], case["phase1"]["claim_points"])
    got = ph1[0]
    assert len(got) == len(ref)
    for (gv, gp), (rv, rp) in zip(got, ref):
        assert gv.tolist() == rv.tolist()
        assert gp.tolist() == rp.tolist()
    assert ph1[3] == 0                     # no check of the reference's failed
    for p, rk in enumerate(case["ranks"]):
        assert sha(ph1[1][p]) == rk["phase1_sha256"]["ip"], p


def test_commit_rows_and_reduction(run):
    case, _, _, _, red, cd = run
    for p, rk in enumerate(case["ranks"]):
        assert sha(cd[p].reshape(-1, 2)) == rk["dealt_sha256"]["commit_data"], p
        h = rk["phase2_sha256"]
        assert (sha(red[0][p]), sha(red[1][p]), sha(red[2][p])) == (h["RA"], h["RB"], h["RC"]), p


def test_phase2_vectors(run):
    case, _, _, ph2, _, _ = run
    vec = ph2[8]
    for p, rk in enumerate(case["ranks"]):
        h = rk["phase2_sha256"]
        assert (sha(vec[0][p]), sha(vec[1][p])) == (h["p1"], h["p2"]), p


def test_phase2_claims_and_ip(run, gbz):
    import gbz_oracle as orc
    import gbz_piop_oracle as po
    case, _, ph1, ph2, _, _ = run
    claims, abc, ip2, ip3, b1, flags, tr, fs = ph2[:8]
    # a, b, c: the three draws after the first phase's coSumcheck
    i = case["draws"].index(ph1[0][0][1][0].tobytes().hex())
    assert [x.tobytes().hex() for x in abc] == case["draws"][i + 1:i + 4]
    ref = ref_claims(case["phase2"]["claims"], case["phase2"]["claim_points"])
    # prove_phase2 returns the second claim's value divided by L_last[0], the
    # Lagrange vector over 2 points at the first phase's last challenge
    # (coPIOP.cpp:434-435, 625); the capture holds the coSumcheck's own value
    L0 = po.lagrange(ph1[0][0][1][-1], 2)[0:1]
    ref[1] = (orc.field_ops(orc.field_ops(L0, L0)[4], ref[1][0].reshape(1, 2))[2][0], ref[1][1])
    assert [(v.tolist(), p.tolist()) for v, p in claims] == [(v.tolist(), p.tolist()) for v, p in ref]
    assert flags == 0
    for p, rk in enumerate(case["ranks"]):
        h = rk["phase2_sha256"]
        assert sha(ip2[p]) == h["ip2"], p
        assert sha(ip3[p]) == h["ip3"], p
    # the chain state: the second coSumcheck's last challenge
    assert fs.tolist() == ref[0][1][0].tolist()
    recs = gbz.parse_transcript(tr)
    assert recs[0][0] == 60
