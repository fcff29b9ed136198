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
