"""libgbz on the host: exports, host-side protocol helpers, transcript layout.

CPU only: nothing here launches a kernel.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, edge_fe, rand_fe


def header_functions():
    src = open(os.path.join(ROOT, "include", "gbz.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbz_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function(gbz):
    names = header_functions()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", gbz.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (gbz_[a-z0-9_]+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert set(gbz.EXPORTS) == set(names)
    for n in names:
        assert hasattr(gbz.lib, n)


def test_host_field_twin_matches_oracle(gbz, oracle):
    rng = np.random.default_rng(5)
    a, b = edge_fe()
    ra, rb = rand_fe(rng, 4000), rand_fe(rng, 4000)
    a, b = np.concatenate([a, ra]), np.concatenate([b, rb])
    s, d, p = gbz.field_ops_host(a, b)
    oa, osub, om, _, _ = oracle.field_ops(a, b)
    assert np.array_equal(s, oa)
    assert np.array_equal(d, osub)
    assert np.array_equal(p, om)


def test_host_fiat_shamir_matches_oracle(gbz, oracle):
    rng = np.random.default_rng(6)
    st1 = np.zeros(2, dtype=np.uint64)
    st2 = np.zeros(2, dtype=np.uint64)
    for k in range(1, 6):
        e = rand_fe(rng, k)
        assert np.array_equal(gbz.hash_to_field(st1, e), oracle.hash_to_field(st2, e))
        assert np.array_equal(st1, st2)


@pytest.mark.parametrize("seed", [0, 1, 42, 3396, 2**32 - 1])
def test_host_prng_matches_oracle(gbz, oracle, seed):
    g1, g2 = gbz.Prng(seed), oracle.Prng(seed)
    for _ in range(50):
        assert np.array_equal(g1.field(), g2.field())
    assert [g1.next() for _ in range(300)] == [g2.next() for _ in range(300)]


@pytest.mark.parametrize("logn,rate", [(3, 2), (4, 4), (5, 2), (6, 4), (9, 8), (10, 2), (13, 4), (16, 2), (18, 4),
                                       (20, 2), (24, 2)])
def test_transcript_layout_matches_oracle(gbz, oracle, logn, rate):
    assert gbz.transcript_bytes(logn, rate) == oracle.transcript_bytes(logn, rate)


def test_transcript_layout_matches_oracle_records(gbz, oracle):
    """Record tags and counts, not only the length (the oracle writes them)."""
    for logn, rate in [(5, 2), (8, 4), (11, 4)]:
        w = oracle.witness(3, 1 << logn)
        t = oracle.prove(w, logn, rate)
        recs = gbz.parse_transcript(t)
        assert sum(8 + len(p) for _, _, p in recs) == len(t) == gbz.transcript_bytes(logn, rate)
        assert recs[0][0] == 1 and recs[-1][0] == 18


def test_invalid_shapes_are_rejected_without_gpu(gbz):
    assert gbz.transcript_bytes(2, 4) == 0      # witness too small
    assert gbz.transcript_bytes(10, 3) == 0     # rate not a power of two
    assert gbz.transcript_bytes(27, 2) == 0     # beyond the supported size
    flat = np.zeros((31, 32), dtype=np.uint8)
    with pytest.raises(gbz.GbzError):
        gbz.open_tree_blake(flat, 64, 16)       # only 16 leaves
    path = gbz.open_tree_blake(flat, 64, 15)
    assert path.shape == (4, 32)


def _gpu_count():
    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        return 0
    n = ctypes.c_int(0)
    return n.value if rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 else 0


def test_context_creation_fails_loudly_without_gpu(gbz):
    if _gpu_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(gbz.GbzError) as e:
        gbz.Context(0)
    assert e.value.status == gbz.ECUDA


def test_missing_library_is_an_import_error(tmp_path, monkeypatch):
    """No CPU fallback: the binding refuses to load without libgbz.so."""
    import importlib.util
    import conftest
    spec = importlib.util.spec_from_file_location("gbz_copy", os.path.join(conftest.PKG, "gbz.py"))
    mod = importlib.util.module_from_spec(spec)
    monkeypatch.setattr(os.path, "exists", lambda p: False if p.endswith("libgbz.so") else True)
    with pytest.raises(ImportError):
        spec.loader.exec_module(mod)


def test_reference_links_against_the_shim(gbz):
    """The drop-in: the reference's own main.cpp and every reference
    translation unit, relinked with host/gbz_reference_shim.cpp and
    libgbz.so in place of the bodies the shim replaces (oracle/ref's
    pigeon_gpu target weakens those definitions in copies of the reference
    objects).  The link must succeed and every function the shim defines
    must resolve to the shim's code in the executable.  It cannot run here
    (no GPU) nor on the GPU host (the reference needs x86-64)."""
    import __graft_entry__
    if not __graft_entry__.reference_dir():
        pytest.skip("reference checkout not available here")
    import build_lib
    lib = os.path.dirname(build_lib.build())
    ref = os.path.join(ROOT, "oracle", "ref")
    r = subprocess.run(["make", "-s", "-j8", "-C", ref, "../_ref/pigeon_gpu", "LIBGBZ=" + lib],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = os.path.join(ROOT, "oracle", "_ref")
    syms = open(os.path.join(out, "shim_symbols.txt")).read().split()
    assert len(syms) >= 15
    # the shim's .text range in the executable, from the link map
    lo = hi = None
    for line in open(os.path.join(out, "pigeon_gpu.map")):
        f = line.split()
        if len(f) >= 4 and f[0].startswith(".text") and f[-1].endswith("shim.o") and f[1].startswith("0x"):
            a0, n = int(f[1], 16), int(f[2], 16)
            lo = a0 if lo is None else min(lo, a0)
            hi = a0 + n if hi is None else max(hi, a0 + n)
    assert lo is not None
    nm = subprocess.run(["nm", os.path.join(out, "pigeon_gpu")], capture_output=True, text=True).stdout
    addr = {}
    for line in nm.splitlines():
        f = line.split()
        if len(f) == 3 and f[1] in "TW":
            addr[f[2]] = int(f[0], 16)
    for s_ in syms + ["random", "rand"]:
        assert lo <= addr[s_] < hi, s_


def test_leader_root_matches_column_merkle(gbz, oracle):
    """gbz_leader_root (host only) equals the leader root that the oracle's
    distributed_MT builds over {root, 0, ..., 0}."""
    rng = np.random.default_rng(5)
    rows = rng.integers(0, (1 << 61) - 1, size=(3, 16, 2), dtype=np.uint64)
    for N in (1, 2, 8, 64):
        levels, root = oracle.column_merkle(rows, N)
        assert np.array_equal(gbz.leader_root(levels[-1], N), root)
