"""The claim of PCS_open_new in the PIOP mode, restated by the oracle, against
the reference's own runs (tests/golden/pcspiop_*.json, written through
oracle/ref's pigeon_dpcs pcs mode by tests/golden/make_golden.py): the
coPCS test's dealing and PCS_commit, the driver's input vectors (Lagrange
vectors at four points of a SplitMix64 stream: b1 over 32 points, b2 the
tensor of two over the row length, b3 over N/4 points) and F_ip with them
(gbz_pcs_oracle.f_ip_vectors), equal to the K the reference's driver passed
to PCS_open_new."""
import json
import os

import numpy as np
import pytest

import conftest

CASES = ["pcspiop_N8_M16.json", "pcspiop_N16_M16.json"]
M64 = (1 << 64) - 1


def load(name):
    with open(os.path.join(conftest.GOLDEN, name)) as f:
        return json.load(f)


def driver_inputs(oracle, N, Bs, seed):
    """The driver's input vectors (oracle/ref/dpcs_mpi_driver.cpp pcs mode)."""
    p = conftest.splitmix_ext((seed * 0x7F4A7C15 + 3) & M64, 4)
    lB = Bs.bit_length() - 1
    la, lb, lk = lB // 2, lB - lB // 2, (N // 4).bit_length() - 1
    La, Lb = oracle.lagrange_coeff(p[1], la), oracle.lagrange_coeff(p[2], lb)
    b2 = oracle.field_ops(np.tile(La, (Lb.shape[0], 1)), np.repeat(Lb, La.shape[0], axis=0))[2]
    return oracle.lagrange_coeff(p[0], 5), b2, oracle.lagrange_coeff(p[3], lk)


@pytest.mark.parametrize("name", CASES)
def test_claim_equals_reference(oracle, name):
    import gbz_pcs_oracle as pcs

    case = load(name)
    N, M = case["N"], 1 << case["logM"]
    sched = pcs.schedule(N, M, case["rates"])
    shares, random = oracle.copcs_party_shares(N, M, sched["randomness"] * N // 4)
    parties = pcs.commit(sched, shares, random)
    Bs = parties[0]["cd"].shape[1]
    b1, b2, b3 = driver_inputs(oracle, N, Bs, case["seed"])
    K = pcs.f_ip_vectors(parties, sched, b1, b2, b3)
    assert np.array(K, dtype=np.uint64).tobytes().hex() == case["K"]


@pytest.mark.parametrize("name", CASES)
def test_schedule_matches_reference_printout(name):
    import gbz_pcs_oracle as pcs

    case = load(name)
    sched = pcs.schedule(case["N"], 1 << case["logM"], case["rates"])
    out = "\n".join(case["stdout"])
    assert "Degrees: " + "".join("%d, " % d for d in sched["degrees"]) in out
    assert "Queries: " + "".join("%d, " % q for q in sched["queries"]) in out
