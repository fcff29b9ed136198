"""The oracle's sumcheck round forms and one-party distributed sumchecks
against the reference's own outputs (fixtures from
oracle/ref/ref_full_driver.cpp via tests/golden/make_golden.py).  CPU only.
"""
import numpy as np
import pytest

from conftest import golden_bytes, splitmix_ext
from test_oracle_copcs import Reader

P = (1 << 61) - 1


def case(golden, name):
    e = golden["sumcheck"][name]
    return Reader(golden_bytes(e["file"])), e["args"]


def feval(coeffs, x):
    """Horner over F_{p^2} in Python integers."""
    acc = (0, 0)
    xr, xi = int(x[0]), int(x[1])
    for c in coeffs:
        acc = ((acc[0] * xr - acc[1] * xi + int(c[0])) % P, (acc[0] * xi + acc[1] * xr + int(c[1])) % P)
    return acc


def fadd(a, b):
    return ((a[0] + b[0]) % P, (a[1] + b[1]) % P)


@pytest.mark.parametrize("name,form", [("zcround_6_0", 3), ("zcround_8_2", 3), ("bround_6_0", 2),
                                       ("bround_7_1", 2)])
def test_round_forms(oracle, golden, name, form):
    r, (_, logm, it, seed) = case(golden, name)
    m = 1 << logm
    raw = splitmix_ext(seed, 6 * m + 2)
    vecs = [raw[k * m:(k + 1) * m] for k in range(6)]
    b, ch = raw[6 * m], raw[6 * m + 1]
    deg = 3 if form == 3 else 2
    H = r.fe(deg + 1)
    half = m >> (it + 1)
    folded = [r.fe(half) for _ in range(6)]
    r.done()
    cur = [v[: m >> it] for v in vecs]
    assert np.array_equal(oracle.sumcheck_round(form, cur, b), H)
    got = oracle.sumcheck_fold_many(cur, ch)
    for g, f in zip(got, folded):
        assert np.array_equal(g, f)


@pytest.mark.parametrize("name", ["cubicsc_8_4", "cubicsc_10_3", "cubicsc_3_4", "quadsc_8_4", "quadsc_11_2"])
def test_party_sumcheck_one_party(oracle, golden, name):
    r, (cmd, logM, offset, seed, prng) = case(golden, name)
    M = 1 << logM
    cubic = cmd == "cubicsc"
    nv = 3 if cubic else 2
    raw = splitmix_ext(seed, nv * M + 1)
    vecs = [raw[k * M:(k + 1) * M] for k in range(nv)]
    w = raw[nv * M:nv * M + 1]
    y = r.fe(1)[0]
    fin = r.fe(nv)
    nr = r.u32()
    chal = r.fe(nr)
    r.done()
    res = oracle.party_sumcheck(1 if cubic else 0, vecs, 1, w=w, offset=offset, prng_seed=prng, y=y)
    assert np.array_equal(res["challenges"], chal)
    assert np.array_equal(res["fin"], fin)
    # every round message is consistent with the running claim
    claim = (int(y[0]), int(y[1]))
    for poly, c in zip(res["polys"], res["challenges"]):
        assert fadd(feval(poly, (0, 0)), feval(poly, (1, 0))) == claim
        claim = feval(poly, c)
    assert claim == (int(res["y"][0]), int(res["y"][1]))


def test_party_sumcheck_many_parties_consistent(oracle):
    """N parties: the aggregated round messages stay consistent with the
    weighted claim sum_p w_p sum_j v1 v2 v3 (cubic) / sum v1 v2 (quadratic)."""
    rng = np.random.default_rng(5)
    N, M = 4, 1 << 7
    for form in (0, 1):
        nv = 3 if form else 2
        vecs = [rng.integers(0, P, size=(N * M, 2), dtype=np.uint64) for _ in range(nv)]
        w = rng.integers(0, P, size=(N, 2), dtype=np.uint64)
        y = (0, 0)
        for p in range(N):
            for j in range(M):
                t = (1, 0)
                for v in vecs:
                    x = v[p * M + j]
                    t = ((t[0] * int(x[0]) - t[1] * int(x[1])) % P, (t[0] * int(x[1]) + t[1] * int(x[0])) % P)
                if form:
                    wp = w[p]
                    t = ((t[0] * int(wp[0]) - t[1] * int(wp[1])) % P, (t[0] * int(wp[1]) + t[1] * int(wp[0])) % P)
                y = fadd(y, t)
        res = oracle.party_sumcheck(form, vecs, N, w=w, offset=3, y=np.array(y, dtype=np.uint64))
        claim = y
        for poly, c in zip(res["polys"], res["challenges"]):
            assert fadd(feval(poly, (0, 0)), feval(poly, (1, 0))) == claim
            claim = feval(poly, c)
        assert len(res["challenges"]) == (7 - 3) + (3 + 2)


def fmul(a, b):
    return ((a[0] * b[0] - a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def quadruple_protocol(round_fn, fold_fn, vecs, y, prng):
    """quadruple_sumcheck (delegate_protocol.cpp:57-115) driven by a round
    function: each round's message must be consistent with the claim, five
    F::_random() draws follow and the last is the challenge.  Returns the
    challenges, the final values and the final claim."""
    cur = vecs
    claim = (int(y[0]), int(y[1]))
    chal = []
    while cur[0].shape[0] > 1:
        H = round_fn(cur)
        assert fadd(feval(H, (0, 0)), feval(H, (1, 0))) == claim
        for _ in range(5):
            r = prng.field()
        chal.append(r)
        claim = feval(H, r)
        cur = fold_fn(cur, r)
    return chal, [c[0] for c in cur], claim


@pytest.mark.parametrize("name", ["quadsc4_6", "quadsc4_9", "quadsc4_1"])
def test_quadruple_sumcheck_vs_reference(oracle, golden, name):
    r, (_, logm, seed, prng) = case(golden, name)
    m = 1 << logm
    raw = splitmix_ext(seed, 4 * m)
    vecs = [raw[k * m:(k + 1) * m] for k in range(4)]
    y = r.fe(1)[0]
    fin = r.fe(4)
    nr = r.u32()
    ref_chal = r.fe(nr)
    r.done()
    chal, finals, claim = quadruple_protocol(lambda cur: oracle.sumcheck_round(4, cur),
                                             lambda cur, c: oracle.sumcheck_fold_many(cur, c),
                                             vecs, y, oracle.Prng(prng))
    assert np.array_equal(np.array(chal, dtype=np.uint64).reshape(-1, 2), ref_chal)
    assert np.array_equal(np.array(finals, dtype=np.uint64).reshape(-1, 2), fin)
    prod = (1, 0)
    for f in finals:
        prod = fmul(prod, (int(f[0]), int(f[1])))
    assert claim == prod
