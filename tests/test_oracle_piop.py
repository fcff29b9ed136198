"""The oracle's restatement of the R1CS front end's dealing and of the data
steps of its two sumcheck phases (oracle/gbz_piop_oracle.py), against what
the unmodified reference computed when its `pigeon 1` ran with N = 8 and 16
ranks (tests/golden/piop_*.json, tests/golden/make_golden.py).

Every rank's dealt inputs, the vectors each phase hands its coSumcheck, the
reduced R1CS matrices, the reshared vector and the inner-product vectors
are compared by SHA-256; the phases' draws, claims and scalars by value.
The coSumchecks themselves are pinned by tests/test_gpu_cosumcheck.py."""
import hashlib
import json
import os

import numpy as np
import pytest

import conftest

CASES = ["piop_N8_M16.json", "piop_N16_M16.json", "piop_N8_M18.json", "piop_N16_M20.json"]
# the restated phase steps loop in Python over every row; the GPU test
# covers the largest case against the same digests
STEPS_MAX_LOGM = 18
RATES = [[4], [4], [4, 4], [4, 4]]


def load(name):
    with open(os.path.join(conftest.GOLDEN, name)) as f:
        return json.load(f)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint64).tobytes()).hexdigest()


def fes(hexes):
    return np.array([[int.from_bytes(bytes.fromhex(h)[:8], "little"), int.from_bytes(bytes.fromhex(h)[8:], "little")]
                     for h in hexes], dtype=np.uint64).reshape(-1, 2)


def claims(blob, points):
    """(value, point) per claim from the fixture's flattened form."""
    v = np.frombuffer(bytes.fromhex(blob), dtype=np.uint64).reshape(-1, 2)
    out, o = [], 0
    for n in points:
        out.append((v[o], v[o + 1:o + 1 + n]))
        o += 1 + n
    return out


@pytest.fixture(scope="module", params=CASES)
def dealt(request, oracle):
    import gbz_piop_oracle as po
    case = load(request.param)
    N, M = case["N"], 1 << case["logM"]
    d = po.deal(N, M, case["generator"]["draws"][0][1], case["pcs_randomness"], case["mask_l"])
    return case, d


def test_dealing(dealt):
    case, d = dealt
    c = d["circuit"]
    assert (c["logm"], c["logn"]) == (case["logm"], case["logn"])
    # the generator positions the reference recorded at generate_sumcheck_randomness
    assert d["counts"]["sumcheck_randomness"] == case["generator"]["draws"][1][1]
    assert (d["degrees1"], d["degrees2"]) == (case["degrees1"], case["degrees2"])
    assert fes([case["K"]])[0].tolist() == [d["K"], 0]
    for p, rk in enumerate(case["ranks"]):
        for key, arr in (("vL", d["vL"]), ("vR", d["vR"]), ("vO", d["vO"]), ("W", d["W"]), ("R1", d["R1"]),
                         ("R2", d["R2"]), ("pcs_random", d["pcs_random"]), ("R", d["R"])):
            assert sha(arr[p]) == rk["dealt_sha256"][key], (p, key)


def test_commit_rows(dealt):
    import gbz_pcs_oracle as pco
    case, d = dealt
    N = case["N"]
    sched = pco.schedule(N, d["W"].shape[1] * N // 4, RATES)
    assert sched["randomness"] == case["pcs_randomness"]
    for p, rk in enumerate(case["ranks"]):
        cd = pco.prepare_data(d["W"][p], d["pcs_random"][p], sched["queries"][0])
        assert [cd.shape[1]] * cd.shape[0] == [x for x in case["commit_rows"] if x], p
        assert sha(cd.reshape(-1, 2)) == rk["dealt_sha256"]["commit_data"], p


def test_phase1_steps(dealt):
    import gbz_oracle as orc
    import gbz_piop_oracle as po
    case, d = dealt
    if case["logM"] > STEPS_MAX_LOGM:
        pytest.skip("covered on the GPU")
    N, k = case["N"], case["N"] // 4
    n = d["vL"].shape[1]
    ln, lk = n.bit_length() - 1, k.bit_length() - 1
    fs0 = fes([case["fs0"]])[0]
    draws, _ = po.fs_draws(fs0, ln + lk + 1)
    assert [x.tobytes().hex() for x in draws] == case["draws"][:ln + lk + 1]
    r1, r2 = np.concatenate([draws[:ln], draws[ln + lk:]]), draws[ln:ln + lk]
    ph = case["phase1"]
    assert fes(ph["r1"]).tolist() == r1.tolist() and fes(ph["r2"]).tolist() == r2.tolist()
    b2 = orc.precompute_beta(r2) if lk else np.array([[1, 0]], dtype=np.uint64)
    # y: each party's masked sum, the leader's interpolation, times the last draw
    ys = []
    for p in range(N):
        m = d["R"][p]
        t = orc.field_ops(orc.field_ops(m[0:4], m[4:8])[2], m[8:12])[1]
        acc = np.zeros((1, 2), dtype=np.uint64)
        for i in range(4):
            acc = orc.field_ops(acc, orc.field_ops(po.beta_index(i, draws[:ln]).reshape(1, 2), t[i:i + 1])[2])[0]
        ys.append(acc[0])
    y = po.unpack_even_dot(np.array(ys), b2)
    y = orc.field_ops(y.reshape(1, 2), r1[-1:])[2][0]
    # K_r: every fourth entry of each round's share of R1, aggregated the same way
    offs = np.cumsum([0] + [4 * x for x in d["degrees1"]])
    kr = []
    for p in range(N):
        acc = np.zeros((1, 2), dtype=np.uint64)
        for a, b in zip(offs[:-1], offs[1:]):
            for v in d["R1"][p][a:b:4]:
                acc = orc.field_ops(acc, v.reshape(1, 2))[0]
        kr.append(acc[0])
    Kr = po.unpack_even_dot(np.array(kr), b2)
    assert fes(ph["K_Kr"]).tolist() == [y.tolist(), Kr.tolist()]
    assert fes([ph["Kr"]])[0].tolist() == Kr.tolist()
    cl = claims(ph["claims"], ph["claim_points"])
    ip = po.ip_vector(cl[0][1][1:], d["degrees1"], 4)
    assert ip.tobytes().hex() == ph["ip"]
    s = po.share_scalars(po.lagrange(cl[0][1][0], N // 4), N)
    for p, rk in enumerate(case["ranks"]):
        for key, v in (("p1", d["vL"]), ("p2", d["vR"]), ("p3", d["vO"])):
            mask = d["R"][p][{"p1": 0, "p2": 4, "p3": 8}[key]:][:4]
            assert sha(po.extend(v[p], mask)) == rk["phase1_sha256"][key], (p, key)
        assert sha(po.scale(ip, s[p])) == rk["phase1_sha256"]["ip"], p


def test_phase2_steps(dealt):
    import gbz_oracle as orc
    import gbz_pcs_oracle as pco
    import gbz_piop_oracle as po
    case, d = dealt
    if case["logM"] > STEPS_MAX_LOGM:
        pytest.skip("covered on the GPU")
    N, k = case["N"], case["N"] // 4
    c1 = claims(case["phase1"]["claims"], case["phase1"]["claim_points"])
    ph = case["phase2"]
    r = c1[0][1]
    assert fes(ph["r"]).tolist() == r[:-1].tolist()
    parts = po.r1cs_rows(d["circuit"], N)
    RA, RB, RC = (po.r1cs_reduce(parts[m], r[:-1], d["degrees1"], case["logm"], N) for m in "ABC")
    # a, b, c: the three draws after the first phase's coSumcheck
    i = case["draws"].index(c1[0][1][0].tobytes().hex())
    a, b, c = fes(case["draws"][i + 1:i + 4])
    L_last = po.lagrange(r[-1], 2)
    lin = lambda x, y, z: orc.field_ops(orc.field_ops(po.scale(x, a), po.scale(y, b))[0], po.scale(z, c))[0]
    aggr = np.stack([po.scale(lin(RA[p], RB[p], RC[p]), L_last[0]) for p in range(N)])
    resh = po.reshare(aggr, N)
    sched = pco.schedule(N, d["W"].shape[1] * N // 4, RATES)
    d1 = d["degrees1"]
    beta = po.tensor([po.lagrange(r[i + 1], d1[i]) for i in range(len(d1) - 1)])
    bsc = po.share_scalars(po.lagrange(r[0], N // 4), N)
    K = orc.field_ops(orc.field_ops(po.scale(c1[0][0].reshape(1, 2), a), po.scale(c1[1][0].reshape(1, 2), b))[0],
                      po.scale(c1[2][0].reshape(1, 2), c))[0][0]
    assert fes(ph["K_Kr"]).tolist() == [K.tolist(), fes([case["K"]])[0].tolist()]
    c2 = claims(ph["claims"], ph["claim_points"])
    ip2 = po.ip_vector(c2[0][1][1:], case["degrees2"], 2)
    assert ip2.tobytes().hex() == ph["ip"]
    s2 = po.share_scalars(po.lagrange(c2[0][1][0], N // 4), N)
    d2 = case["degrees2"]
    L = po.lagrange(c2[0][1][1], d2[0])
    for i in range(1, len(d2)):
        L = po.scale(L, po.lagrange(c2[0][1][i + 1], d2[i])[0])
    for p, rk in enumerate(case["ranks"]):
        h = rk["phase2_sha256"]
        assert (sha(RA[p]), sha(RB[p]), sha(RC[p])) == (h["RA"], h["RB"], h["RC"]), p
        assert sha(aggr[p]) == h["R_aggr"], p
        assert sha(resh[p]) == h["reshared"], p
        bs = po.scale(po.scale(beta, bsc[p]), L_last[1])
        bs = np.concatenate([bs, np.zeros((3 * bs.shape[0], 2), dtype=np.uint64)])
        assert sha(np.concatenate([po.segment_aggr(resh[p], case["mask_l"]), bs])) == h["p2"], p
        cd = pco.prepare_data(d["W"][p], d["pcs_random"][p], sched["queries"][0])
        rows = [cd[j] for j in range(cd.shape[0])] + [np.zeros((0, 2), dtype=np.uint64)] * (
            len(case["commit_rows"]) - cd.shape[0])
        w = po.witness_layout(rows, max(case["commit_rows"]), case["mask_l"])
        m = d["R"][p]
        rl = np.zeros_like(w)
        rl[:4] = lin(m[0:4], m[4:8], m[8:12])
        assert sha(np.concatenate([w, rl])) == h["p1"], p
        assert sha(po.scale(ip2, s2[p])) == h["ip2"], p
        ip3 = np.concatenate([po.scale(L[:4], a), po.scale(L[:4], b), po.scale(L[:4], c)])
        assert sha(po.scale(ip3, s2[p])) == h["ip3"], p
