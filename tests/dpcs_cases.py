"""Inputs of the distributed-PCS fixtures (tests/golden/dpcs.json): rank p's
arrays as oracle/ref/dpcs_mpi_driver.cpp draws them (SplitMix64 seeded with
the case seed and p, arr then arr2)."""
import numpy as np

import conftest

M64 = (1 << 64) - 1


def driver_arrays(case):
    N, A = case["N"], 1 << case["logA"]
    two = case["mode"] == "batch"
    arr, arr2 = [], []
    for p in range(N):
        raw = conftest.splitmix_ext((case["seed"] * 0x10001 + p * 0x9E3779B1 + 11) & M64, (2 if two else 1) * A)
        arr.append(raw[:A])
        if two:
            arr2.append(raw[A:])
    return np.stack(arr), (np.stack(arr2) if two else None)


def column_height(N):
    lN = N.bit_length() - 1
    return 1 << (lN - lN // 2)


def open_inputs(case, oracle_mod):
    """The inputs the driver's open mode builds (dpcs_mpi_driver.cpp
    open_mode): per polynomial l the parties' arrays (arr2 zero for l > 0),
    their global codeword rows (the interleaved transform), the point r_l
    from the stream all ranks share and the claim y_l."""
    import gbz_dpcs_oracle as do
    P, N, A, nb, rate, seed = case["P"], case["N"], 1 << case["logA"], case["batch"], case["rate"], case["seed"]
    S, L = A // nb, A // nb * rate
    lS, lR, lN = S.bit_length() - 1, (nb - 1).bit_length(), N.bit_length() - 1
    shared = conftest.splitmix_ext((seed * 0x7F4A7C15 + 3) & M64, P * (lS + lR + lN))
    cd, cwg, arrs_all, r, y = [], [], [], [], []
    for l in range(P):
        arrs, arr2s = [], []
        for p in range(N):
            raw = conftest.splitmix_ext((seed * 0x10001 + p * 0x9E3779B1 + 11 + 0x1000 * l) & M64, 2 * A)
            arrs.append(raw[:A])
            a2 = raw[A:].copy()
            if l > 0:
                a2[:] = 0
            arr2s.append(a2)
        arrs = np.stack(arrs)
        arrs_all.append(arrs)
        cd.append([a.reshape(nb, S, 2) for a in arr2s])
        rows = []
        for k in range(nb):
            G = np.zeros((N * L, 2), dtype=np.uint64)
            for p in range(N):
                G[p:N * S:N] = arrs[p, k * S:(k + 1) * S]
            rows.append(oracle_mod.fft(G))
        cwg.append(np.stack(rows))
        rl = shared[l * (lS + lR + lN):(l + 1) * (lS + lR + lN)]
        r.append(rl)
        b2 = oracle_mod.precompute_beta(rl[:lS])
        b3 = oracle_mod.precompute_beta(rl[lS:lS + lR])
        b1 = oracle_mod.precompute_beta(rl[lS + lR:])
        acc = np.zeros(2, dtype=np.uint64)
        for p in range(N):
            v = oracle_mod.field_ops(do._dot_vec(b2, do._sum_rows(cd[l][p], b3)).reshape(1, 2), b1[p:p + 1])[2][0]
            acc = oracle_mod.field_ops(acc.reshape(1, 2), v.reshape(1, 2))[0][0]
        y.append(acc)
    return cd, cwg, arrs_all, r, y


def query_count(rate):
    import math
    return int(-100.0 / math.log2(math.sqrt(1.0 / rate)))
