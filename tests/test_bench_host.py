"""Host-side pieces of bench.py: the work and byte models the rooflines
divide by, and the clock sampler's fallbacks (no GPU needed)."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_commit_lengths_halve(bench):
    ls = bench.commit_lengths(24, 2)
    assert ls[0] == 1 << 25 and ls[1] == 1 << 24
    assert all(a == 2 * b for a, b in zip(ls, ls[1:]))
    assert len(ls) == 12  # the witness commitment and 11 WHIR re-encodings


def test_work_model(bench):
    w = bench.algorithmic_int_work(24, 2)
    # witness commitment as a real-input transform of half length M = 2^24
    M = 1 << 24
    first = M // 2 * 24 + M
    rest = sum(L // 2 * (L.bit_length() - 1) for L in bench.commit_lengths(24, 2)[1:])
    assert w["ntt"] == first + rest
    # roots (depth + 1 each) plus l depth (depth + 1) / 2 per opened codeword
    assert 100_000 < w["merkle_chain"] < 200_000


def test_byte_model(bench):
    b = bench.algorithmic_bytes(24, 2)
    n = 1 << 24
    assert b["beta"] == 16 * (n // 2) + 16 * (n // 4)
    assert b["ntt"] > 16 * n + 16 * 2 * n  # at least the witness read and its codeword written
    assert set(b) == {"sumcheck", "ntt", "beta", "update_betas"}


def test_clock_sampler_without_nvml_or_smi(bench, monkeypatch):
    """Neither NVML nor nvidia-smi (as in a container without a driver):
    the sampler reports no samples instead of failing."""
    monkeypatch.setattr(bench.ClockSampler, "_nvml_open", lambda self: None)
    monkeypatch.setenv("PATH", "/nonexistent")
    with bench.ClockSampler(0) as clk:
        pass
    s = clk.summary()
    assert s["samples"] == 0 and s["sm_mhz"] is None and s["reasons"] == []
