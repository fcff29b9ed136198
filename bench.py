#!/usr/bin/env python3
"""Throughput of the plain single-party prover on GB300.

Workload (one step = one proof): a 2^24-evaluation witness of uniform
base-field values (SplitMix64, seed 0x5EEF0000), Reed-Solomon rate 1/2
(codeword 2^25), Blake3 Merkle tree over the codeword, quadratic sumcheck
with Fiat-Shamir challenges, WHIR opening with folding factor 4 until at
most 4 coefficients remain.  Every step emits the full transcript, which is
checked against the CPU oracle once per run.

Prints one JSON line:
  value        proofs/s with the witness resident in HBM (device pointers)
  e2e          proofs/s through the public API with pinned HOST buffers:
               the K steps as one gbz_prove_batch call (3 slots), every
               step's witness H2D copy and transcript D2H copy inside the
               timed region; single_call beside it is one synchronised
               gbz_prove per step (per-proof latency p50/p99)
  roofline     the dominant kernel category, timed with CUDA events on the
               launching stream during a second timed pass
  cpu_baseline the oracle port (oracle/gbz_oracle.c) proving the same
               workload once on the host cores
  batched      64 proofs (2^12..2^20, rate 1/4) through
               gbz_prove_batch (8 slots, graph replay; grouped: the proofs
               of each shape share every launch, and per proof for
               comparison) beside the plain prover (one synchronised
               gbz_prove per proof), same pinned host buffers, transcripts
               compared byte for byte
  served       400 Poisson arrivals at 200/s (2^14..2^22,
               rate 1/2 or 1/4) through gbz_serve: proofs/s, p50/p99
               latency, beside the plain prover on the same arrivals; and
               both at saturation (every request at t = 0)
  --impl reference: the reference arm.  The reference's CPU prover does not
               build on the Arm GPU host (x86-64 inline asm in
               fieldElement.cpp), so this arm times the oracle port, which is
               pinned byte for byte to the reference's transcripts.

Multi-GPU: proofs are independent, so N GPUs run N replicas (weak scaling,
no collective); `value` sums the proofs of all ranks over the slowest rank's
time.
"""
import argparse
import hashlib
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "shorter-and-faster-post-quantum-secure-scalable-collaborative-snarks_gb300")
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)
sys.path.insert(0, ORACLE)

LOGN, RATE = 24, 2
# DRAM bytes of every transform launch of one proof (both passes of each
# transform, the packed pass and the unpack), from one ncu capture of the
# n = 2^22 proof (dram__bytes_read.sum, dram__bytes_write.sum, kernels
# ntt_pass_kernel and real_unpack_kernel, four proofs within 0.3 %); scaled
# by n for other sizes (the later, smaller transforms' writes stay in L2 at
# 2^22, so the write figure is a lower bound).
NTT_TRAFFIC_2E22 = {"read": 585.3e6, "write": 175.0e6}
E2E_LANES = 3  # slots of the batched end-to-end pass
SERVE_REPEATS = 3  # interleaved repeats of the served and plain runs at 200 requests/s
SEED = 0x5EED0000 + 2 * 65536  # witness seed of the 2^24 rate-1/2 workload
METRIC = "proofs/s and p50/p99 latency, batched+served vs plain GPU prover, bit-exact"
CONFIG = {
    "workload": "plain prover, n=2^24 uniform base-field witness, rate 1/2 (NTT 2^25), Blake3 Merkle over "
                "2^23 leaves of 4 elements, FS sumcheck (24 rounds), WHIR folding 4 (11 iterations)",
    "logn": LOGN, "rate": RATE, "whir_k": 4,
    "l2": "inputs larger than L2 (witness 256 MiB, codeword 512 MiB per step)",
}

# Algorithmic bytes per proof by kernel category: what each category must read and write at least.
def algorithmic_bytes(logn, rate):
    n, L = 1 << logn, (1 << logn) * rate
    out = {}
    # main sumcheck (eq-factored): round 0 reads w and the eq table E_0
    # (n/2 entries); every fold at length m reads w_i and E_i (m/2) and
    # writes w_{i+1} (m/2) and E_{i+1} (m/4): 36 m bytes
    sc = 16 * n + 8 * n
    m = n
    while m > 1:
        sc += 36 * m
        m //= 2
    # WHIR: both rounds of an iteration in one pass, reading arr and b and
    # writing the quarter-length pair (40 m bytes); the first iteration reads
    # the eq table of chal[2..] (m/4 entries) instead of b (28 m bytes)
    m, wsc = n, 0
    while m > 4:
        wsc += (16 * m + 4 * m + 8 * m) if m == n else 40 * m
        m //= 4
    out["sumcheck"] = sc + wsc
    # NTT: read valid input + write codeword, per commit.  (The prover's
    # Merkle work is chains of compressions from single leaves, latency
    # bound; the whole-tree kernel is measured as a row.)
    ntt = 16 * n + 16 * L
    m, cur = n, rate
    while m > 4:
        m //= 4
        NL = 2 * cur * m
        ntt += 16 * m + 16 * NL
        cur *= 2
    out["ntt"] = ntt
    out["beta"] = 16 * (n // 2) + 16 * (n // 4)  # E_0 of z_1.. and E_2 of chal[2..], written once
    m, cur, ub = n, rate, 0
    while m > 4:
        m //= 4
        ub += 2 * 16 * m
        cur *= 2
    out["update_betas"] = ub
    return out


def commit_lengths(logn, rate):
    """Codeword lengths of every commitment of one proof (initial + WHIR)."""
    n = 1 << logn
    out = [n * rate]
    m, cur = n, rate
    while m > 4:
        m //= 4
        out.append(2 * cur * m)
        cur *= 2
    return out


def algorithmic_int_work(logn, rate):
    """Integer-pipe work per proof: radix-2 butterfly count (L/2 log2 L) of
    the commitment transforms (the witness commitment is a base-field
    transform, done as a half-length transform of packed pairs plus one
    multiply per output pair: M/2 log2 M + M for M = L/2), and the Blake3
    compressions of the Merkle
    nodes the proof reveals (inner nodes hash their left child twice, so the
    root is a chain of depth + 1 compressions from leaf 0 and path entry d a
    chain of d + 1 from one leaf): root chains plus l depth (depth + 1) / 2
    per opened codeword."""
    ls = commit_lengths(logn, rate)
    comps = 0
    for k, L in enumerate(ls):  # codeword k has rate rate * 2^k
        depth = (L // 4).bit_length() - 1
        comps += depth + 1
        if k + 1 < len(ls):  # every codeword but the last is opened
            l = int(-100 / np.log2(np.sqrt(1.0 / (rate << k))))
            comps += l * depth * (depth + 1) // 2
    M = ls[0] // 2
    ntt = M // 2 * (M.bit_length() - 1) + M + sum(L // 2 * (L.bit_length() - 1) for L in ls[1:])
    return {"ntt": ntt, "merkle_chain": comps, "update_betas": update_betas_fmuls(logn, rate)}


def update_betas_fmuls(logn, rate):
    """F_{p^2} multiplies of the WHIR beta updates of one proof, as the prover
    runs them (gbz_prover.cu: update_betas_by_transform).  Iteration t adds
    sum_i c_i w^{q_i j} (l queries) to the m new entries of b, with the
    exponents taken at half the new codeword length T = NL / 2: when l m >
    4 T (and T > 2^13) as one second pass of a length-T transform whose rows
    are formed from the entries (T / N1 rows of N1 = 2^k1, k1 = ceil(log2 T
    / 2): 3 multiplies per (entry, row) to form them, (N1 / 2) k1
    butterflies per row), else as direct geometric sums (l m)."""
    n = 1 << logn
    m, cur, total = n, rate, 0
    while m > 4:
        l = int(-100 / np.log2(np.sqrt(1.0 / cur)))
        m //= 4
        NL = 2 * cur * m
        T = NL // 2
        lt = T.bit_length() - 1
        if 13 < lt <= 26 and m <= T and l * m > 4 * T:
            k1 = (lt + 1) // 2
            total += 3 * l * (T >> k1) + (T // 2) * k1
        else:
            total += l * m
        cur *= 2
    return total


class ClockSampler:
    """SM clocks and throttle reasons sampled during the timed region: NVML
    queries (read only) every 5 ms from a thread, or nvidia-smi's 200 ms
    loop when the NVML library cannot be loaded."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock event reason bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, device):
        self.device, self.proc, self.lines = device, None, []
        self.nvml, self.samples, self.max_mhz, self.stop = None, [], None, threading.Event()

    def _nvml_open(self):
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = ctypes.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.device), ctypes.byref(h)) != 0:
                return None
            mx = ctypes.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:  # NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
            fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            return lib, h, fn
        except (OSError, AttributeError):
            return None

    def _nvml_loop(self):
        lib, h, reasons_fn = self.nvml
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0:
                r = rs.value if reasons_fn(h, ctypes.byref(rs)) == 0 else 0
                self.samples.append((float(clk.value), r))
            time.sleep(0.005)

    def __enter__(self):
        self.nvml = self._nvml_open()
        if self.nvml:
            self.t = threading.Thread(target=self._nvml_loop, daemon=True)
            self.t.start()
            deadline = time.time() + 1.0
            while not self.samples and time.time() < deadline:  # sampling before the region starts
                time.sleep(0.002)
            self.samples.clear()  # keep only samples taken inside the region
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.nvml:
            self.stop.set()
            self.t.join(timeout=1)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.nvml:
            reasons = sorted({nm for _, r in self.samples for bit, nm in self.REASONS.items() if r & bit})
            return {"sm_mhz": statistics.median([c for c, _ in self.samples]) if self.samples else None,
                    "sm_max_mhz": self.max_mhz, "reasons": reasons, "samples": len(self.samples),
                    "source": "NVML, 5 ms"}
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi, 200 ms"}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return ws, rank, local


def barrier_and_max(value, ws):
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference_arm(args, ws, rank):
    """The reference arm: the oracle port on all host cores, same workload."""
    if rank != 0:
        return
    import gbz_oracle as O
    O.build()
    w = O.witness(SEED, 1 << LOGN)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.prove(w, LOGN, RATE, 1, threads=cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.prove(w, LOGN, RATE, 1, threads=cores)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "proofs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (F_{p^2}, p=2^61-1)",
        "data": "synthetic", "config": dict(CONFIG, parallelism="replicas%d" % args.gpus),
        "p50_ms": 1e3 * float(np.percentile(times, 50)), "p99_ms": 1e3 * float(np.percentile(times, 99)),
        "cpu_baseline": {"value": value, "unit": "proofs/s", "cores": cores, "kind": "port",
                         "sample": "full proofs of the same workload (oracle/gbz_oracle.c, pthreads)"},
        "e2e": {"value": value, "unit": "proofs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own CPU code needs x86-64 (inline mulx asm, AVX types) and does not build on the "
                "Arm host; the port reproduces its transcripts byte for byte",
    }
    print(json.dumps(line), flush=True)


def c3_jobs():
    """The batch workload: 64 witnesses, log2 n uniform in [12, 20], rate 1/4."""
    rng = np.random.default_rng(0x5EEF3)
    return [int(x) for x in rng.integers(12, 21, size=64)], [4] * 64


def c5_requests(n_req, lam, seed=0x5EEF5):
    """The serving workload: Poisson arrivals (rate lam per second), log2 n uniform
    in [14, 22], rate 1/2 or 1/4."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / lam, size=n_req))
    arrivals -= arrivals[0]
    logns = [int(x) for x in rng.integers(14, 23, size=n_req)]
    rates = [int(x) for x in rng.choice([2, 4], size=n_req)]
    return arrivals, logns, rates


def run_many(gbz, O, ctx, repeats, served=True):
    """Batched (C3) and served (C5) proving against the plain prover (one
    gbz_prove call per proof, synchronised) on the same jobs, pinned host
    buffers, transcripts compared byte for byte."""
    out = {}
    pinned = {}

    def witness(logn, cfg):
        key = (logn, cfg)
        if key not in pinned:
            p = gbz.PinnedArray((1 << logn, 2), np.uint64)
            p.array[...] = O.witness(0x5EED0000 + cfg * 65536 + logn, 1 << logn)
            pinned[key] = p
        return pinned[key].array

    def transcripts(logns, rates):
        bufs = [gbz.PinnedArray((gbz.transcript_bytes(l, r),), np.uint8) for l, r in zip(logns, rates)]
        return bufs, [b.array for b in bufs]

    # ---- C3: batch
    logns, rates = c3_jobs()
    ws = [witness(l, 3) for l in logns]
    seeds = list(range(1, len(logns) + 1))
    keep, tb = transcripts(logns, rates)
    for w, l, r, s, t in zip(ws, logns, rates, seeds, tb):
        ctx.prove(w, l, r, s, out=t)
    t0 = time.perf_counter()
    for _ in range(repeats):
        for w, l, r, s, t in zip(ws, logns, rates, seeds, tb):
            ctx.prove(w, l, r, s, out=t)
    plain = len(ws) * repeats / (time.perf_counter() - t0)
    ref = [t.tobytes() for t in tb]
    keep2, tb2 = transcripts(logns, rates)

    def batch_rate(grouped):
        ctx.set_grouping(grouped)
        ctx.prove_batch(ws, logns, rates, seeds, lanes=8, out=tb2)
        mks = []
        t0 = time.perf_counter()
        for _ in range(repeats):
            _, lat, mk = ctx.prove_batch(ws, logns, rates, seeds, lanes=8, out=tb2)
            mks.append(mk)
        rate = len(ws) * repeats / (time.perf_counter() - t0)
        return rate, min(mks), [t.tobytes() for t in tb2] == ref

    # per proof: one plan and graph replay per proof on 8 slots
    ungrouped, mk_u, same_u = batch_rate(False)
    # grouped (the default): the proofs of each shape share every launch
    batched, mk_g, same_g = batch_rate(True)
    out["batched"] = {
        "workload": "64 proofs, n = 2^12..2^20 log-uniform, rate 1/4",
        "proofs_per_s": batched, "plain_proofs_per_s": plain, "speedup_vs_plain": batched / plain,
        "device_makespan_ms": 1e3 * mk_g, "slots": 8, "graphs": True, "grouped": True,
        "ungrouped_proofs_per_s": ungrouped, "ungrouped_makespan_ms": 1e3 * mk_u,
        "bit_identical_to_plain": same_g and same_u,
    }
    if not served:
        return out
    # ---- C5: serving at 200 requests/s, and at saturation (all at once)
    arrivals, slog, srate = c5_requests(400, 200.0)
    sws = [witness(l, 5) for l in slog]
    sseeds = list(range(1, len(slog) + 1))
    keep3, st3 = transcripts(slog, srate)
    ctx.prove_batch(sws, slog, srate, sseeds, lanes=8, out=st3)  # warm plans and graphs
    served = {}
    # served and plain interleaved over SERVE_REPEATS repeats of the same
    # arrivals (plain: one proof at a time, each replayed from its graph like
    # gbz_prove); the median of each figure with its spread (min, max)
    runs = {}
    for _ in range(SERVE_REPEATS):
        for name, arr, kw in [("served", arrivals, dict(lanes=8, depth=2)),
                              ("plain", arrivals, dict(lanes=1, depth=1))]:
            _, lat, mk = ctx.serve(arr, sws, slog, srate, sseeds, out=st3, **kw)
            runs.setdefault(name, []).append((len(slog) / mk, 1e3 * float(np.percentile(lat, 50)),
                                              1e3 * float(np.percentile(lat, 99))))
    for name, rs in runs.items():
        a = np.array(rs)
        served[name] = {"proofs_per_s": float(np.median(a[:, 0])), "p50_ms": float(np.median(a[:, 1])),
                        "p99_ms": float(np.median(a[:, 2])),
                        "p50_ms_range": [float(a[:, 1].min()), float(a[:, 1].max())],
                        "p99_ms_range": [float(a[:, 2].min()), float(a[:, 2].max())], "repeats": len(rs)}
    for name, arr, kw in [("served_saturated", np.zeros(len(slog)), dict(lanes=8, depth=2)),
                          ("plain_saturated", np.zeros(len(slog)), dict(lanes=1, depth=1))]:
        _, lat, mk = ctx.serve(arr, sws, slog, srate, sseeds, out=st3, **kw)
        served[name] = {"proofs_per_s": len(slog) / mk, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                        "p99_ms": 1e3 * float(np.percentile(lat, 99))}
    sref = []
    for w, l, r, s in zip(sws[:32], slog[:32], srate[:32], sseeds[:32]):
        sref.append(ctx.prove(w, l, r, s).tobytes())
    out["served"] = {
        "workload": "400 requests, Poisson 200/s, n = 2^14..2^22 log-uniform, rate 1/2 or 1/4",
        "slots": 8, "depth": 2, **served,
        "bit_identical_to_alone": [t.tobytes() for t in st3[:32]] == sref,
    }
    return out


PCS_RATES = [[4], [4], [4, 4], [4, 4]]  # the reference's coPCS test (main.cpp:54)


def pcs_point(gbz, n):
    """The opening point of the coPCS test: hash_to_field({0}) n times from a
    fresh chain (main.cpp:83-85); returns (r, chain state)."""
    fs = np.zeros(2, dtype=np.uint64)
    r = []
    for _ in range(n):
        fs = gbz.hash_to_field(fs, np.zeros((1, 2), dtype=np.uint64))
        r.append(fs.copy())
    return np.array(r, dtype=np.uint64), fs


def run_party_shares(gbz, O, ctx, repeats, N=16, logM=24):
    """Configuration 4: the reference's coPCS test (main.cpp:49-163) with
    N = 16 parties on one device, M = 2^24 shared coefficients (2^22 share
    entries per party): PCS_commit, the claim (F_ip) and PCS_open_new, once
    up to the leader's delegation (gbz_pcs_open) and once whole
    (gbz_pcs_open_full: the leader's delegation proofs, final checks and
    WHIR opening too), all device resident (torch buffers, C-ABI calls on
    device pointers).  The shares are the ones the reference's rank 0 deals
    (glibc's default stream, generated on the host before timing); the
    transcripts are compared with the reference's own 16-rank run when its
    fixture is present (tests/golden/parties_N16_M24.json)."""
    import torch
    M = 1 << logM
    deg, q, rnd = gbz.pcs_schedule(N, M, PCS_RATES)
    shares, random, g_deal = O.copcs_party_shares(N, M, rnd * N // 4, state=True)
    sh = torch.from_numpy(shares.view(np.int64)).cuda()
    rn = torch.from_numpy(random.view(np.int64)).cuda()
    r0 = np.array([x[0] for x in PCS_RATES], dtype=np.int32)
    r1 = np.array([x[1] if len(x) > 1 else 0 for x in PCS_RATES], dtype=np.int32)
    r, fs0 = pcs_point(gbz, logM + 1)
    rd = torch.from_numpy(r.view(np.int64)).cuda()
    Kd = torch.zeros(2, dtype=torch.int64, device="cuda")
    fsd = torch.zeros(2, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    lib = gbz.lib

    def commit():
        h = ctypes.c_void_p()
        ctx.check(lib.gbz_pcs_commit(ctx.h, N, M, len(PCS_RATES), r0.ctypes.data, r1.ctypes.data, sh.data_ptr(),
                                     rn.data_ptr(), gbz.MEM_DEVICE, ctypes.byref(h), None, None))
        return h

    def open_(h, tr):
        ctx.check(lib.gbz_pcs_claim(ctx.h, h, rd.data_ptr(), r.shape[0], Kd.data_ptr(), gbz.MEM_DEVICE))
        fsd.copy_(torch.from_numpy(fs0.view(np.int64)))
        ctx.check(lib.gbz_pcs_open(ctx.h, h, rd.data_ptr(), r.shape[0], Kd.data_ptr(), fsd.data_ptr(),
                                   tr.data_ptr(), tr.numel(), gbz.MEM_DEVICE))
        ctx.synchronize()

    # the whole of PCS_open_new: the leader's tail draws from rank 0's
    # generator as the dealing leaves it
    flags = ctypes.c_uint32(0)

    def open_full(h, trf):
        g = gbz.Prng(1)
        ctypes.memmove(ctypes.addressof(g), g_deal, ctypes.sizeof(g))
        ctx.check(lib.gbz_pcs_claim(ctx.h, h, rd.data_ptr(), r.shape[0], Kd.data_ptr(), gbz.MEM_DEVICE))
        fsd.copy_(torch.from_numpy(fs0.view(np.int64)))
        ctx.check(lib.gbz_pcs_open_full(ctx.h, h, rd.data_ptr(), r.shape[0], Kd.data_ptr(), fsd.data_ptr(),
                                        ctypes.addressof(g), ctypes.byref(flags), trf.data_ptr(), trf.numel(),
                                        gbz.MEM_DEVICE))
        ctx.synchronize()

    h = commit()
    nbytes, fbytes = ctypes.c_uint64(0), ctypes.c_uint64(0)
    ctx.check(lib.gbz_pcs_info(h, None, None, None, ctypes.byref(nbytes)))
    ctx.check(lib.gbz_pcs_open_full_bytes(h, ctypes.byref(fbytes)))
    tr = torch.zeros(nbytes.value, dtype=torch.uint8, device="cuda")
    trf = torch.zeros(fbytes.value, dtype=torch.uint8, device="cuda")
    open_(h, tr)  # warm-up (checked on the device: GBZ_ECHECK otherwise)
    open_full(h, trf)
    lib.gbz_pcs_free(h)
    t_c, t_o, t_f = [], [], []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = commit()
        t1 = time.perf_counter()
        open_(h, tr)
        t2 = time.perf_counter()
        open_full(h, trf)
        t3 = time.perf_counter()
        lib.gbz_pcs_free(h)
        t_c.append(t1 - t0)
        t_o.append(t2 - t1)
        t_f.append(t3 - t2)
    digest = hashlib.sha256(tr.cpu().numpy().tobytes()).hexdigest()
    full = gbz.parse_transcript(trf.cpu().numpy().tobytes())
    # PCS_open_new in the PIOP mode (isPIOP = true, as coPIOP_prove calls
    # it) on the same commitment: b1, b2 = La x Lb and b3 Lagrange vectors
    # at seeded points, their claim from gbz_pcs_claim_piop, the WHIR slots
    # left on the device
    h = commit()
    rl = ctypes.c_uint64(0)
    ctx.check(lib.gbz_pcs_info(h, None, ctypes.byref(rl), None, None))
    Bs = rl.value
    lB = Bs.bit_length() - 1
    pts = O.witness(0x9107, 4)
    b1 = O.lagrange_coeff(pts[0], 5)
    La, Lb = O.lagrange_coeff(pts[1], lB // 2), O.lagrange_coeff(pts[2], lB - lB // 2)
    b3 = O.lagrange_coeff(pts[3], (N // 4).bit_length() - 1)
    b2 = O.field_ops(np.tile(La, (Lb.shape[0], 1)), np.repeat(Lb, La.shape[0], axis=0))[2]
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()
    db1, db2, db3, dlag = dv(b1), dv(b2), dv(b3), dv(np.concatenate([La, Lb]))
    logs = (ctypes.c_int * 2)(lB // 2, lB - lB // 2)
    pbytes = ctypes.c_uint64(0)
    ctx.check(lib.gbz_pcs_open_piop_bytes(h, logs, 2, ctypes.byref(pbytes), None))
    trp = torch.zeros(pbytes.value, dtype=torch.uint8, device="cuda")
    pflags = ctypes.c_uint32(0)

    def open_piop():
        g = gbz.Prng(1)
        ctypes.memmove(ctypes.addressof(g), g_deal, ctypes.sizeof(g))
        ctx.check(lib.gbz_pcs_claim_piop(ctx.h, h, db1.data_ptr(), 32, db2.data_ptr(), Bs, db3.data_ptr(), N // 4,
                                         Kd.data_ptr(), gbz.MEM_DEVICE))
        fsd.zero_()
        ctx.check(lib.gbz_pcs_open_piop(ctx.h, h, db1.data_ptr(), 32, db2.data_ptr(), Bs, db3.data_ptr(), N // 4,
                                        dlag.data_ptr(), logs, 2, Kd.data_ptr(), fsd.data_ptr(), ctypes.addressof(g),
                                        ctypes.byref(pflags), None, trp.data_ptr(), trp.numel(), gbz.MEM_DEVICE))
        ctx.synchronize()

    open_piop()
    t_p = []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        open_piop()
        t_p.append(time.perf_counter() - t0)
    lib.gbz_pcs_free(h)
    out = {"workload": "the reference's coPCS test (PCS_commit + F_ip + PCS_open_new; open_full adds the "
                       "leader's delegation proofs, final checks and WHIR opening) with %d parties on one device, "
                       "M = 2^%d (2^%d share entries per party), "
                       "rates {{4},{4},{4,4},{4,4}}" % (N, logM, logM + 2 - (N.bit_length() - 1)),
           "parties": N, "share_len": 4 * M // N, "degrees": deg, "queries": q,
           "commit_ms": 1e3 * min(t_c), "open_ms": 1e3 * min(t_o), "total_ms": 1e3 * (min(t_c) + min(t_o)),
           "runs_per_s": 1.0 / (min(t_c) + min(t_o)), "transcript_bytes": int(nbytes.value),
           "transcript_sha256": digest,
           "open_full_ms": 1e3 * min(t_f), "full_total_ms": 1e3 * (min(t_c) + min(t_f)),
           "full_runs_per_s": 1.0 / (min(t_c) + min(t_f)), "full_transcript_bytes": int(fbytes.value),
           "leader_flags": int(flags.value),
           "open_piop_ms": 1e3 * min(t_p), "open_piop_flags": int(pflags.value),
           "open_piop_workload": "PCS_open_new with isPIOP (gbz_pcs_claim_piop + gbz_pcs_open_piop): Lagrange input "
                                 "vectors, the WHIR batch slots and delegate_lagrange_eval instead of the aggregated "
                                 "opening and delegate_beta_eval",
           "timing": "host wall clock around the synchronised C-ABI calls (device pointers), best of %d" % repeats}
    tx = os.path.join(ROOT, "tests", "golden", "dpcs_timing.json")
    if os.path.exists(tx):
        with open(tx) as f:
            pp = json.load(f).get("pcs_piop", {})
        if (pp.get("N"), pp.get("logM")) == (N, logM):
            # the reference's PCS_open_new(..., true) at this size, 16 ranks on an
            # 8-core x86 host (recorded by tests/golden/make_golden.py)
            out["open_piop_reference_seconds_x86"] = pp["open_seconds"]
    fx = os.path.join(ROOT, "tests", "golden", "parties_N%d_M%d.json" % (N, logM))
    if os.path.exists(fx):
        with open(fx) as f:
            ref = json.load(f)
        out["transcript_equals_reference"] = ref.get("gpu_transcript_sha256") == digest
        out["reference_ranks_seconds_x86"] = ref.get("ref_seconds")
        lead = ref.get("leader")
        if lead:
            # the leader's tail against rank 0's records: the segments'
            # commitment roots, the delegation claims, the WHIR opening's
            # final claim and the beta delegation's claim
            tags = lambda t: [p for k, _, p in full if k == t]
            ok = [x.hex() for x in tags(46)] == [rd["root"] for rd in lead["rounds"]]
            ok &= [x.hex() for x in tags(52)] == [rd["pex"] for rd in lead["rounds"]]
            ok &= all(c.hex().startswith(rd["pmf"]) for c, rd in zip(tags(50), lead["rounds"]))
            ok &= tags(54)[0].hex() == lead["whir_claim"] and tags(56)[0].hex() == lead["beta_eval_y"]
            out["leader_tail_equals_reference"] = bool(ok)
    return {"party_shares": out}


def run_dpcs(gbz, O, ctx, repeats, N=16, logA=20, batch=16, rate=4):
    """The distributed PCS's batch commitment (Batch_dCommit,
    distributed_PCS.cpp:56-147) of 16 parties on one device: 2^20 entries
    per party in 16 rows, rate 4 (coPIOP's witness_commit_rate), so 16
    transforms of length N L = 2^22 (the reference's distributed FFT), the
    column hashes and 16 trees of 2^18 leaves; device pointers, host clock
    around the synchronised call, best of `repeats`."""
    import torch
    A = 1 << logA
    arr = torch.from_numpy(O.witness(0xD9C5, N * A).view(np.int64).reshape(N, A, 2)).cuda()
    arr2 = torch.from_numpy(O.witness(0xD9C6, N * A).view(np.int64).reshape(N, A, 2)).cuda()
    L = A // batch * rate
    cd = torch.empty_like(arr2)
    cw = torch.empty((N, batch, L, 2), dtype=torch.int64, device="cuda")
    lv = torch.empty((N, 2 * L - 1, 32), dtype=torch.uint8, device="cuda")
    roots = np.zeros((N, 32), dtype=np.uint8)
    lead = np.zeros(32, dtype=np.uint8)
    torch.cuda.synchronize()

    def call():
        ctx.check(gbz.lib.gbz_dpcs_batch_commit(ctx.h, N, A, arr.data_ptr(), arr2.data_ptr(), rate, batch,
                                                cd.data_ptr(), cw.data_ptr(), lv.data_ptr(), roots.ctypes.data,
                                                lead.ctypes.data, gbz.MEM_DEVICE))
    call()
    ts = []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        call()
        ts.append(time.perf_counter() - t0)
    t = min(ts)
    # algorithmic bytes: every party's arr read, arr2 copied (read + write),
    # the codewords written and read for the columns, the trees written
    moved = 16 * N * A * 3 + 2 * 16 * N * batch * L + 32 * N * (2 * L - 1)
    # the opening (PIOP_dOpen_batch_new) of this commitment with a second one
    # of zero data, as coPIOP_prove opens the witness with the index
    cw2 = torch.empty_like(cw)
    zero = torch.zeros_like(arr2)
    ctx.check(gbz.lib.gbz_dpcs_batch_commit(ctx.h, N, A, arr.data_ptr(), zero.data_ptr(), rate, batch, None,
                                            cw2.data_ptr(), None, None, None, gbz.MEM_DEVICE))
    S = A // batch
    cds = torch.stack([arr2.reshape(N, batch, S, 2), zero.reshape(N, batch, S, 2)]).contiguous()
    cws = torch.stack([cw, cw2]).contiguous()
    lS, lR, lN = S.bit_length() - 1, batch.bit_length() - 1, N.bit_length() - 1
    pts = torch.from_numpy(O.witness(0xD9C7, 2 * (lS + lR + lN)).view(np.int64)).cuda()
    ys = torch.zeros((2, 2), dtype=torch.int64, device="cuda")
    fsd = torch.zeros(2, dtype=torch.int64, device="cuda")
    nb = gbz.lib.gbz_dpcs_open_bytes(N, 2, rate)
    tr = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    fl = ctypes.c_uint32(0)

    def open_():
        fsd.zero_()
        torch.cuda.synchronize()
        ctx.check(gbz.lib.gbz_dpcs_open(ctx.h, N, 2, batch, S, rate, cds.data_ptr(), cws.data_ptr(), pts.data_ptr(),
                                        ys.data_ptr(), 0, rate, fsd.data_ptr(), None, None, None, None, None,
                                        ctypes.byref(fl), tr.data_ptr(), nb, gbz.MEM_DEVICE))
    open_()
    to = []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        open_()
        to.append(time.perf_counter() - t0)
    ref = {}
    fx = os.path.join(ROOT, "tests", "golden", "dpcs_timing.json")
    if os.path.exists(fx) and (N, logA, batch, rate) == (16, 20, 16, 4):
        with open(fx) as f:
            rj = json.load(f)
        # the reference's Batch_dCommit and PIOP_dOpen_batch_new at this size,
        # 16 ranks on an 8-core x86 host (recorded by tests/golden/make_golden.py)
        ref = {"reference_ranks_seconds_x86": {"commit": rj["commit_seconds"], "open": rj["open_seconds"],
                                               "ranks": rj["ranks"], "host_cores": rj["host_cores"]}}
    return {"dpcs": dict(ref, **{"open_ms": 1e3 * min(to),
                     "open_workload": "PIOP_dOpen_batch_new of the witness commitment and a zero index commitment "
                                      "(2 x 16 rows of 2^%d per party), unchecked claims" % (lS,),
                     "workload": "Batch_dCommit of %d parties, 2^%d entries each in %d rows, rate %d: %d transforms "
                                 "of length 2^%d, %d trees of 2^%d leaves" % (N, logA, batch, rate, batch,
                                                                              (N * L).bit_length() - 1, N,
                                                                              L.bit_length() - 1),
                     "ms": 1e3 * t, "commits_per_s": 1.0 / t, "bytes_moved": moved, "gbs": moved / t / 1e9,
                     "timing": "host wall clock around the synchronised C-ABI call (device pointers), best of %d"
                               % repeats})}


def run_piop(gbz, O, ctx, repeats, N=16, logM=20):
    """The R1CS front end's two sumcheck phases (pigeon 1: prove_phase1 and
    prove_phase2, coPIOP.cpp:241-627) with N = 16 parties on one device and
    a circuit of M = 2^20 gates, every input device resident: the parties'
    shares as rank 0 deals them (regenerated on the host before timing), the
    witness laid out from gbz_pcs_commit's rows, the R1CS rows uploaded once.
    Timed: gbz_piop_phase1 then gbz_piop_phase2 (host clock around the
    synchronised calls, best of `repeats`).  Both phases' claims are compared
    with the reference's own 16-rank run when its fixture is present
    (tests/golden/piop_N16_M20.json)."""
    import torch
    import gbz_piop_oracle as po
    M = 1 << logM
    fx = os.path.join(ROOT, "tests", "golden", "piop_N%d_M%d.json" % (N, logM))
    ref = json.load(open(fx)) if os.path.exists(fx) else None
    circ = po.circuit(M)
    mask_l = 333   # (int)(100 / -log2(1 - 0.25 (1 - 1/4))) (coPIOP.cpp:1392-1393)
    k = N // 4
    nW = (1 << circ["logn"]) // k
    deg, q, rnd = gbz.pcs_schedule(N, nW * N // 4, PCS_RATES)
    d = po.deal(N, M, circ["draws"], rnd, mask_l)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()
    vL, vR, vO, R1, R2 = (dev(d[x]) for x in ("vL", "vR", "vO", "R1", "R2"))
    masks = dev(d["R"][:, :12])
    com, _, _ = gbz.pcs_commit(ctx, N, nW * N // 4, PCS_RATES, d["W"], d["pcs_random"])
    w = []
    for p in range(N):
        rows, _, _ = com.data(p)
        lst = [rows[j] for j in range(rows.shape[0])] + [np.zeros((0, 2), dtype=np.uint64)] * (32 - rows.shape[0])
        w.append(po.witness_layout(lst, com.row_len, mask_l))
    com.free()
    w = np.stack(w)
    nw = w.shape[1]
    wd = dev(w)
    parts = po.r1cs_rows(circ, N)
    ptrs, cols = [], []
    for m in "ABC":
        pp, cc, base = [np.zeros(1, dtype=np.int64)], [], 0
        for ptr, c in parts[m]:
            pp.append(ptr[1:] + base)
            cc.append(c)
            base += c.shape[0]
        ptrs.append(np.concatenate(pp))
        cols.append(np.concatenate(cc))
    r1cs = gbz.R1cs(ctx, N, (1 << circ["logn"]) // N, circ["logm"], ptrs, cols)
    d1 = np.array(d["degrees1"], dtype=np.int32)
    d2 = np.array(d["degrees2"], dtype=np.int32)
    fs0 = np.zeros(2, dtype=np.uint64) if ref is None else np.frombuffer(bytes.fromhex(ref["fs0"]), dtype=np.uint64)
    K = np.array([d["K"], 0], dtype=np.uint64)
    n = d["vL"].shape[1]
    lib = gbz.lib
    b1_bytes = lib.gbz_piop_phase1_bytes(N, n, d1.ctypes.data, len(d1))
    b2_bytes = lib.gbz_piop_phase2_bytes(N, d2.ctypes.data, len(d2))
    tr1 = torch.zeros(b1_bytes, dtype=torch.uint8, device="cuda")
    tr2 = torch.zeros(b2_bytes, dtype=torch.uint8, device="cuda")
    cl1 = torch.zeros((4, len(d1) + 2, 2), dtype=torch.int64, device="cuda")
    cl2 = torch.zeros((5, len(d2) + 2, 2), dtype=torch.int64, device="cuda")
    ip1 = torch.zeros((N, 4 * int(d1.sum()), 2), dtype=torch.int64, device="cuda")
    ip2 = torch.zeros((N, 2 * int(d2.sum()), 2), dtype=torch.int64, device="cuda")
    ip3 = torch.zeros((N, 12, 2), dtype=torch.int64, device="cuda")
    abc = torch.zeros((3, 2), dtype=torch.int64, device="cuda")
    fsd = torch.zeros(2, dtype=torch.int64, device="cuda")
    Kd = dev(K)
    fl1, fl2 = ctypes.c_uint32(0), ctypes.c_uint32(0)

    def phases():
        fsd.copy_(torch.from_numpy(fs0.view(np.int64)))
        torch.cuda.synchronize()
        ctx.check(lib.gbz_piop_phase1(ctx.h, N, n, vL.data_ptr(), vR.data_ptr(), vO.data_ptr(), masks.data_ptr(),
                                      R1.data_ptr(), d1.ctypes.data, len(d1), fsd.data_ptr(), cl1.data_ptr(),
                                      ip1.data_ptr(), None, None, ctypes.byref(fl1), tr1.data_ptr(), b1_bytes,
                                      gbz.MEM_DEVICE))
        point1 = cl1[0, 1:].contiguous()
        evals1 = cl1[:3, 0].contiguous()
        torch.cuda.synchronize()
        ctx.check(lib.gbz_piop_phase2(ctx.h, N, nw, wd.data_ptr(), masks.data_ptr(), r1cs.h, mask_l, R2.data_ptr(),
                                      point1.data_ptr(), evals1.data_ptr(), d1.ctypes.data, len(d1), d2.ctypes.data,
                                      len(d2), Kd.data_ptr(), fsd.data_ptr(), cl2.data_ptr(), abc.data_ptr(),
                                      ip2.data_ptr(), ip3.data_ptr(), None, None, ctypes.byref(fl2),
                                      tr2.data_ptr(), b2_bytes, gbz.MEM_DEVICE))

    phases()  # warm-up (pools, twiddle tables)
    ts = []
    for _ in range(repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        phases()
        ts.append(time.perf_counter() - t0)
    r1cs.free()
    out = {"workload": "the R1CS front end's first and second sumcheck (prove_phase1 + prove_phase2) of %d parties "
                       "on one device, circuit of M = 2^%d gates (pigeon 1's random circuit), vL/vR/vO 2^%d and "
                       "witness 2^%d entries per party" % (N, logM, n.bit_length() - 1, nw.bit_length() - 1),
           "parties": N, "degrees1": d["degrees1"], "degrees2": d["degrees2"],
           "phases_ms": 1e3 * min(ts), "runs_per_s": 1.0 / min(ts), "flags": [fl1.value, fl2.value],
           "timing": "host wall clock around the synchronised C-ABI calls (device pointers), best of %d" % repeats}
    if ref is not None:
        def blob(t, rows):
            a = t.cpu().numpy().astype(np.uint64)
            v = []
            for i in range(rows):
                v.append(a[i, 0])
                v.extend(a[i, 1:])
            return np.array(v, dtype=np.uint64).tobytes().hex()
        c2 = cl2.cpu().numpy().astype(np.uint64).copy()
        # prove_phase2 divides the second claim by L_last[0]; the fixture holds the coSumcheck's own
        out["claims_equal_reference"] = (blob(cl1, 4) == ref["phase1"]["claims"] and
                                         c2[0].tobytes().hex() == bytes.fromhex(ref["phase2"]["claims"])[
                                             :16 * (len(d2) + 2)].hex())
        out["reference_ranks_seconds_x86"] = ref.get("ref_seconds")
    return {"piop": out}


def run_rows(gbz, ctx, rt, stream, fmul_peak, b3_peak, hbm_peak, shift=0):
    """One device-resident measurement per hot-path row outside the plain
    prover: CUDA events on the context's stream around each C-ABI call
    (best of 3 after a warm-up), with the algorithmic work of the call and
    its roofline fraction (HBM bytes, or F_{p^2} multiplies / Blake3
    compressions against the measured integer peaks).  shift divides every
    size by 2^shift (small cases for profiler captures)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(7)
    P61 = (1 << 61) - 1

    def rnd(n):  # canonical random field elements on the device
        return torch.randint(0, P61, (n, 2), dtype=torch.int64, device="cuda", generator=g)

    ev = []
    for _ in range(2):
        e = ctypes.c_void_p()
        assert rt.cudaEventCreate(ctypes.byref(e)) == 0
        ev.append(e)

    def timed(fn):
        fn()
        ctx.synchronize()
        best = 1e30
        for _ in range(3):
            rt.cudaEventRecord(ev[0], stream)
            fn()
            rt.cudaEventRecord(ev[1], stream)
            rt.cudaEventSynchronize(ev[1])
            x = ctypes.c_float()
            rt.cudaEventElapsedTime(ctypes.byref(x), ev[0], ev[1])
            best = min(best, x.value)
        return best

    rows = {}

    def rec(name, ms, hbm_bytes=None, fmuls=None, comps=None, note=""):
        r = {"ms": ms}
        t = ms / 1e3
        if hbm_bytes:
            r["hbm_gbs"] = hbm_bytes / t / 1e9
            r["hbm_frac"] = r["hbm_gbs"] / hbm_peak
        if fmuls:
            r["g_fmul_s"] = fmuls / t / 1e9
            r["int_frac"] = fmuls / t / fmul_peak
        if comps:
            r["g_blake3_s"] = comps / t / 1e9
            r["int_frac"] = comps / t / b3_peak
        if note:
            r["work"] = note
        rows[name] = r

    D = gbz.MEM_DEVICE
    # 16-party cubic distributed sumcheck over 2^24 entries (fused fold + message per round)
    N, M = 16, 1 << (20 - shift)
    v = [rnd(N * M) for _ in range(3)]
    w = np.ascontiguousarray(np.random.default_rng(1).integers(0, P61, size=(N, 2), dtype=np.uint64))
    nr = gbz.lib.gbz_party_sumcheck_rounds(M, N, 4)
    polys, chal, fin = gbz.fe_array(4 * nr), gbz.fe_array(nr), gbz.fe_array(3)
    fs, yy = np.zeros(2, np.uint64), np.zeros(2, np.uint64)

    def party():
        pr = gbz.Prng(1)
        gbz.lib.gbz_party_sumcheck(ctx.h, gbz.SC_CUBIC, v[0].data_ptr(), v[1].data_ptr(), v[2].data_ptr(), M, N,
                                   gbz._ptr(w), 4, gbz._ptr(fs), ctypes.addressof(pr), gbz._ptr(yy),
                                   gbz._ptr(polys), gbz._ptr(chal), gbz._ptr(fin), D)  # y = 0: ECHECK, timed all the same
    m, byts = N * M, 0
    byts += 3 * 16 * m
    # cubic message of a pair: 3 + 6 products (linear x linear, then x linear);
    # a fused round folds 4 entries of each vector (6) and adds one pair (9)
    fm = 9 * (m // 2)
    while m >= 4:
        byts += 3 * 16 * m + 3 * 16 * (m // 2)
        fm += 15 * (m // 4)
        m //= 2
    rec("party_sumcheck_cubic_2^%d" % (24 - shift), timed(party), hbm_bytes=byts, fmuls=fm,
        note="16 parties x 2^%d, 3 vectors" % (20 - shift))
    del v
    # coPCS Encode, 16 rows of 2^20 at rate 2
    R, lr = 16, 20 - shift
    rows_in, cw = rnd(R << lr), torch.empty(((R << lr) * 2, 2), dtype=torch.int64, device="cuda")
    enc = lambda: ctx.check(gbz.lib.gbz_encode_rows(ctx.h, rows_in.data_ptr(), R, lr, 2, 0, cw.data_ptr(), D))
    # rate 2, offset 0: the inverse transform and one length-n coset transform
    # (the codeword's odd positions are the row itself), n coset multiplies
    bfly = R * (2 * ((1 << lr) // 2 * lr) + (1 << lr))
    rec("encode_rows_16x2^%d_rate2" % lr, timed(enc), fmuls=bfly,
        note="radix-2 butterflies of the inverse and the half-length coset transform, plus the coset shift")
    # whole Blake3 Merkle tree (the drop-in MT_commit_Blake) over a 2^25 codeword
    lt = 25 - shift
    cwt = rnd(1 << lt)
    lvt = torch.empty(((1 << lt) // 2 - 1, 32), dtype=torch.uint8, device="cuda")
    mt = lambda: ctx.check(gbz.lib.gbz_merkle_commit_blake(ctx.h, cwt.data_ptr(), 1 << lt, lvt.data_ptr(), D))
    rec("merkle_tree_2^%d" % lt, timed(mt), hbm_bytes=16 * (1 << lt) + 32 * ((1 << lt) // 2 - 1),
        comps=(1 << lt) // 2 - 1, note="2^%d leaves of 4 elements + every inner node" % (lt - 2))
    del cwt, lvt
    # column Merkle over 32 rows of 2^20
    lc = 20 - shift
    cols = rnd(32 << lc)
    lv = torch.empty(((2 << lc) - 1, 32), dtype=torch.uint8, device="cuda")
    root = torch.empty(32, dtype=torch.uint8, device="cuda")
    cm = lambda: ctx.check(gbz.lib.gbz_column_merkle(ctx.h, cols.data_ptr(), 32, lc, 16, lv.data_ptr(),
                                                     root.data_ptr(), D))
    rec("column_merkle_32x2^%d" % lc, timed(cm), comps=4 * (1 << lc) + (1 << lc) - 1,
        note="4 compressions per column + tree over 2^20 column roots")
    del cols, lv
    # RS_multifold5 of a 2^24 codeword by 16
    lm = 24 - shift
    cwb = rnd(1 << lm)
    a16 = np.ascontiguousarray(np.random.default_rng(2).integers(0, P61, size=(16, 2), dtype=np.uint64))
    mf = torch.empty((1 << (lm - 4), 2), dtype=torch.int64, device="cuda")
    mfc = lambda: ctx.check(gbz.lib.gbz_rs_multifold5(ctx.h, cwb.data_ptr(), 1 << lm, gbz._ptr(a16), 4,
                                                      mf.data_ptr(), D))
    # per output: 4 butterfly levels of 8 (32 products), 15 twiddles + 3 squarings, 16 Lagrange weights, d^-1
    rec("rs_multifold5_2^%d_by16" % lm, timed(mfc), hbm_bytes=16 * (1 << lm) + 16 * (1 << (lm - 4)),
        fmuls=67 * (1 << (lm - 4)), note="integer-ALU bound: 67 F-muls per output")
    # coSumcheck phase 2 (fold by Lagrange weights), 2^24 by 16
    c2 = lambda: ctx.check(gbz.lib.gbz_cosumcheck_phase2(ctx.h, cwb.data_ptr(), 1 << lm, gbz._ptr(a16), 4,
                                                         mf.data_ptr(), D))
    rec("cosumcheck_phase2_2^%d_d16" % lm, timed(c2), hbm_bytes=16 * (1 << lm) + 16 * (1 << (lm - 4)))
    # coSumcheck phase 1, cubic, 2^22 per vector, blocks of 8
    l1 = 22 - shift
    p4 = [rnd(1 << l1) for _ in range(4)]
    H = np.zeros((32, 2), dtype=np.uint64)
    c1 = lambda: ctx.check(gbz.lib.gbz_cosumcheck_phase1(ctx.h, p4[0].data_ptr(), p4[1].data_ptr(),
                                                         p4[2].data_ptr(), p4[3].data_ptr(), 1 << l1, 3,
                                                         gbz._ptr(H), D))
    nb = (1 << l1) // 8
    rec("cosumcheck_phase1_cubic_2^%d_d8" % l1, timed(c1),
        fmuls=4 * nb * (8 // 2 * 3 + 32 // 2 * 5) + 3 * nb * 32, note="block transforms (butterflies) + products")
    del p4
    # packed Shamir shares, 2^22 values for 16 parties
    ls = 22 - shift
    sv = rnd(1 << ls)
    sh = torch.empty((16, (1 << ls) // 4, 2), dtype=torch.int64, device="cuda")
    ssh = lambda: ctx.check(gbz.lib.gbz_secret_shares(ctx.h, sv.data_ptr(), 1 << ls, 16, 0, 1, sh.data_ptr(), D))
    rec("secret_shares_2^%d_N16" % ls, timed(ssh), fmuls=((1 << ls) // 4) * 16 * 8,
        hbm_bytes=16 * (1 << ls) + 16 * 16 * ((1 << ls) // 4))
    # leader aggregation of 64 party messages of 2^16
    msgs = rnd(64 << 16)
    bb = np.ascontiguousarray(np.random.default_rng(3).integers(0, P61, size=(16, 2), dtype=np.uint64))
    ao = torch.empty((1 << 16, 2), dtype=torch.int64, device="cuda")
    ag = lambda: ctx.check(gbz.lib.gbz_party_aggregate(ctx.h, msgs.data_ptr(), 64, 1 << 16, gbz._ptr(bb),
                                                       ao.data_ptr(), D))
    # the length-2^25 transform with the first pass's twiddles read from the
    # full table (the prover's default) against formed on the fly from the
    # two-level table: the same values, one multiply per element more
    L25 = 1 << (25 - shift)
    xs = rnd(L25)
    lg25 = L25.bit_length() - 1
    ffull = lambda: ctx.check(gbz.lib.gbz_fft(ctx.h, xs.data_ptr(), lg25, 0, D))
    t_full = timed(ffull)
    gbz.lib.gbz_ntt_full_twiddles(0)
    t_fly = timed(ffull)
    gbz.lib.gbz_ntt_full_twiddles(1)
    bfl = L25 // 2 * lg25
    rec("ntt_2^25_full_twiddle_table", t_full, fmuls=bfl, note="radix-2 butterfly count; first-pass twiddles "
        "read from the full table (the prover's default)")
    rec("ntt_2^25_twiddles_on_the_fly", t_fly, fmuls=bfl, note="the same transform with the first-pass twiddles "
        "formed from the two-level table (one more multiply per element, 134 MB less read)")
    rec("party_aggregate_64x2^16", timed(ag), hbm_bytes=16 * (65 << 16),
        note="the 64-point unpack-and-weight map built on the device (one CTA) then one pass over the "
             "messages; host call incl. the 16 weights' copy")
    # aggregate_claims, 4 arrays x 4 points of 2^22
    la = 22 - shift
    arrs = [rnd(1 << la) for _ in range(4)]
    pts = np.ascontiguousarray(np.random.default_rng(4).integers(0, P61, size=(4, la, 2), dtype=np.uint64))
    oa = torch.empty((1 << la, 2), dtype=torch.int64, device="cuda")
    ob = torch.empty((1 << la, 2), dtype=torch.int64, device="cuda")
    K, ch = np.zeros(2, np.uint64), gbz.fe_array(8)
    plist = (ctypes.c_void_p * 4)(*[a.data_ptr() for a in arrs])

    def aggc():
        pr = gbz.Prng(1)
        ctx.check(gbz.lib.gbz_whir_aggregate_claims(ctx.h, 4, ctypes.cast(plist, ctypes.c_void_p), 1 << la, 4,
                                                    gbz._ptr(pts), ctypes.addressof(pr), oa.data_ptr(),
                                                    ob.data_ptr(), gbz._ptr(K), gbz._ptr(ch), None, D))
    n22 = 16 << la
    rec("whir_aggregate_claims_4x4_2^%d" % la, timed(aggc),
        hbm_bytes=(4 + 2) * n22,  # the arrays read once, b_aggr and arr written
        fmuls=(4 + 16 + 8) * (1 << la),  # eq entries, 4 x 4 inner products, two 4-term combinations
        note="eq tables formed on the fly from half-length tables (never written), 16 inner products and "
             "2 combinations in two passes of two points over the 4 arrays")
    del arrs, msgs
    # pcs_sumcheck_phase3, 2^20 rows, 100 queries, 16 parties
    lb = 20 - shift
    Bv = rnd(1 << lb)
    qs = np.ascontiguousarray(np.stack([np.random.default_rng(5).integers(0, 8, 100),
                                        np.random.default_rng(6).integers(0, 2 << lb, 100)], 1).astype(np.uint32))
    s3 = np.array([12345, 678], dtype=np.uint64)
    ph3 = lambda: ctx.check(gbz.lib.gbz_pcs_sumcheck_phase3(ctx.h, Bv.data_ptr(), 1 << lb, gbz._ptr(qs), 100,
                                                            gbz._ptr(s3), 16, 2, 3, D))
    rec("pcs_phase3_2^%d_l100" % lb, timed(ph3), note="geometric update of 100 terms over 2^%d rows" % lb)
    del Bv
    # Whir_Batch_Open of three polynomials of 2^22, 2^20, 2^18 at rate 1/2 (folding 4), device resident
    logs = [22 - shift, 20 - shift, 18 - shift]
    sizes = [1 << x for x in logs]
    sch = gbz.whir_batch_schedule(sizes, 2, 4)
    if sch is not None:
        barr = [rnd(x) for x in sizes]
        bet = []
        for x in logs:
            pt = rnd(x)
            b = torch.empty((1 << x, 2), dtype=torch.int64, device="cuda")
            ctx.check(gbz.lib.gbz_precompute_beta(ctx.h, pt.data_ptr(), x, b.data_ptr(), D))
            bet.append(b)
        cws = []
        lv0 = None
        for i, (a, L) in enumerate(zip(barr, sch[2])):
            c = torch.empty((L, 2), dtype=torch.int64, device="cuda")
            lv = torch.empty((L // 2 - 1, 32), dtype=torch.uint8, device="cuda")
            ctx.check(gbz.lib.gbz_whir_commit(ctx.h, a.data_ptr(), a.shape[0], L // a.shape[0], c.data_ptr(),
                                              lv.data_ptr(), D))
            cws.append(c)
            if i == 0:
                lv0 = lv
        h = ctx.sumcheck_round(gbz.SC_QUADRATIC, [barr[0], bet[0]])
        K0 = np.array([(int(h[0][k]) + int(h[1][k]) + 2 * int(h[2][k])) % P61 for k in (0, 1)], dtype=np.uint64)
        ctx.whir_batch_open(barr, cws, lv0, bet, K0, 2, 4, prng=1)  # checked on the device (GBZ_ECHECK otherwise)
        bo = lambda: ctx.whir_batch_open(barr, cws, lv0, bet, K0, 2, 4, prng=1)
        rec("whir_batch_open_2^%d_2^%d_2^%d_rate2" % tuple(logs), timed(bo),
            note="Whir_Batch_Open: %d schedule steps, 2 merges, %d transcript bytes (host call incl. planning "
                 "and the final synchronisation)" % (len(sch[0]), sch[3]))
    return {"rows": rows}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbz", choices=["gbz", "reference"])
    ap.add_argument("--logn", type=int, default=LOGN)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-many", action="store_true", help="skip the batched and served measurements")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default NTT and Merkle shapes")
    ap.add_argument("--rows-only", action="store_true", help="only the per-row measurements (profiling)")
    ap.add_argument("--rows-shift", type=int, default=0, help="divide the per-row sizes by 2^k")
    ap.add_argument("--parties-only", action="store_true", help="only the party-shares (coPCS) measurement")
    ap.add_argument("--parties-repeats", type=int, default=3, help="timed repeats of the party-shares run")
    ap.add_argument("--batch-only", action="store_true", help="only the batched (64 mixed proofs) measurement")
    ap.add_argument("--piop-only", action="store_true",
                    help="only the R1CS front end's two sumcheck phases and the distributed PCS commitment")
    ap.add_argument("--batch-repeats", type=int, default=3, help="timed repeats of the batched measurement")
    args = ap.parse_args()
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
        return

    import build_lib
    build_lib.build()
    import gbz
    import gbz_oracle as O
    O.build()
    logn = args.logn
    n = 1 << logn
    w = O.witness(SEED + rank, n)  # each replica proves its own witness
    tbytes = gbz.transcript_bytes(logn, RATE)
    launches = gbz.prove_launches(logn, RATE)

    ctx = gbz.Context(local)
    rt = ctypes.CDLL("libcudart.so")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaEventCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
    rt.cudaEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    rt.cudaEventSynchronize.argtypes = [ctypes.c_void_p]
    rt.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
    stream = gbz.lib.gbz_get_stream(ctx.h)

    if args.parties_only:
        print(json.dumps(run_party_shares(gbz, O, ctx, repeats=args.parties_repeats)), flush=True)
        ctx.close()
        return
    if args.batch_only:
        print(json.dumps(run_many(gbz, O, ctx, args.batch_repeats, served=False)), flush=True)
        ctx.close()
        return
    if args.piop_only:
        out = run_piop(gbz, O, ctx, repeats=3)
        out.update(run_dpcs(gbz, O, ctx, repeats=3))
        print(json.dumps(out), flush=True)
        ctx.close()
        return

    if args.rows_only:
        fmul_peak, b3_peak = ctx.calibrate()
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                hbm = float(json.load(f)["hbm_gbs"])
        except (OSError, KeyError, ValueError):
            hbm = 6800.0
        print(json.dumps(run_rows(gbz, ctx, rt, stream, fmul_peak, b3_peak, hbm, args.rows_shift)), flush=True)
        ctx.close()
        return

    # device-resident witness and transcript
    dw, dt = ctypes.c_void_p(), ctypes.c_void_p()
    ctx.check(gbz.lib.gbz_device_alloc(ctx.h, ctypes.byref(dw), w.nbytes))
    ctx.check(gbz.lib.gbz_device_alloc(ctx.h, ctypes.byref(dt), tbytes))
    assert rt.cudaMemcpy(dw, w.ctypes.data, w.nbytes, 1) == 0

    def prove_device():
        ctx.check(gbz.lib.gbz_prove(ctx.h, dw, logn, RATE, 1, dt, tbytes, gbz.MEM_DEVICE))

    def events(k):
        evs = []
        for _ in range(k):
            e = ctypes.c_void_p()
            assert rt.cudaEventCreate(ctypes.byref(e)) == 0
            evs.append(e)
        return evs

    # autotuning of the transform shapes and the Merkle level fusion for the
    # lengths this proof commits to (identical results for every choice)
    tuned = {}
    if not args.no_autotune:
        t0 = time.perf_counter()
        for L in commit_lengths(logn, RATE):
            lg = L.bit_length() - 1
            if lg > 13:
                sh, ms_d, ms_b = ctx.ntt_autotune(lg, reps=3)
                tuned["ntt_2^%d" % lg] = {"shape": sh, "ms_default": ms_d, "ms_best": ms_b}
        lgm, ms_d, ms_b = ctx.merkle_autotune((commit_lengths(logn, RATE)[0]).bit_length() - 1, reps=3)
        tuned["merkle"] = {"log_nodes_per_cta": lgm, "ms_default": ms_d, "ms_best": ms_b}
        tuned["seconds"] = time.perf_counter() - t0

    # correctness: the device transcript equals the oracle's
    prove_device()
    ctx.synchronize()
    got = np.zeros(tbytes, dtype=np.uint8)
    assert rt.cudaMemcpy(got.ctypes.data, dt, tbytes, 2) == 0

    for _ in range(args.warmup):
        prove_device()
    ctx.synchronize()

    # timed pass 1: device-resident inputs
    ev = events(args.steps + 1)
    with ClockSampler(local) as clk:
        rt.cudaEventRecord(ev[0], stream)
        for i in range(args.steps):
            prove_device()
            rt.cudaEventRecord(ev[i + 1], stream)
        rt.cudaEventSynchronize(ev[-1])
    lat = []
    for i in range(args.steps):
        x = ctypes.c_float()
        rt.cudaEventElapsedTime(ctypes.byref(x), ev[i], ev[i + 1])
        lat.append(x.value)
    total_ms = sum(lat)
    total_ms = barrier_and_max(total_ms, ws)
    value = ws * args.steps / (total_ms / 1e3)

    # timed pass 2: per-category kernel time with events on the same stream
    ctx.profile_enable(True)
    ctx.profile_read(logn, RATE)
    for _ in range(args.steps):
        prove_device()
    ctx.synchronize()
    prof = ctx.profile_read(logn, RATE)
    ctx.profile_enable(False)

    # timed pass 3: end to end through the public API with pinned host buffers
    hw_p, ht_p = ctypes.c_void_p(), ctypes.c_void_p()
    ctx.check(gbz.lib.gbz_host_alloc(ctypes.byref(hw_p), w.nbytes))
    ctx.check(gbz.lib.gbz_host_alloc(ctypes.byref(ht_p), tbytes))
    ctypes.memmove(hw_p, w.ctypes.data, w.nbytes)
    for _ in range(2):
        ctx.check(gbz.lib.gbz_prove(ctx.h, hw_p, logn, RATE, 1, ht_p, tbytes, gbz.MEM_HOST))
    t0 = time.perf_counter()
    e2e_lat = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        ctx.check(gbz.lib.gbz_prove(ctx.h, hw_p, logn, RATE, 1, ht_p, tbytes, gbz.MEM_HOST))
        e2e_lat.append(time.perf_counter() - t1)
    e2e_s = time.perf_counter() - t0
    e2e_s = barrier_and_max(e2e_s, ws)
    e2e = ws * args.steps / e2e_s
    host_t = np.ctypeslib.as_array(ctypes.cast(ht_p, ctypes.POINTER(ctypes.c_uint8)), shape=(tbytes,)).copy()
    assert host_t.tobytes() == got.tobytes()

    # timed pass 4: end to end through gbz_prove_batch, the public call for
    # many proofs: the K steps are one batch over E2E_LANES slots with the
    # same pinned host buffers, so each step's witness upload and transcript
    # read overlap other proofs' work (the upload runs at the host link's
    # ~210 GB/s whichever engine moves it)
    hw_view = np.ctypeslib.as_array(ctypes.cast(hw_p, ctypes.POINTER(ctypes.c_uint64)), shape=(n, 2))
    touts = [gbz.PinnedArray((tbytes,), np.uint8) for _ in range(args.steps)]
    warm = min(E2E_LANES, args.steps)
    ctx.prove_batch([hw_view] * warm, [logn] * warm, [RATE] * warm, [1] * warm, lanes=E2E_LANES,
                    out=[t.array for t in touts[:warm]])
    t0 = time.perf_counter()
    ctx.prove_batch([hw_view] * args.steps, [logn] * args.steps, [RATE] * args.steps, [1] * args.steps,
                    lanes=E2E_LANES, out=[t.array for t in touts])
    batch_s = barrier_and_max(time.perf_counter() - t0, ws)
    e2e_batch = ws * args.steps / batch_s
    assert all(t.array.tobytes() == got.tobytes() for t in touts)
    del touts
    ctx.sched_release()

    # rooflines per kernel category: HBM for the streaming kernels, the
    # measured integer-pipe peaks for the NTT (F_{p^2} multiplies) and the
    # Merkle levels (Blake3 compressions)
    algo = algorithmic_bytes(logn, RATE)
    work = algorithmic_int_work(logn, RATE)
    per_proof_ms = {k: v[0] / args.steps for k, v in prof.items()}
    dom = max(per_proof_ms, key=lambda k: per_proof_ms[k])
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak, peak_src = float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        hbm_peak, peak_src = 6800.0, "fallback"
    fmul_peak, b3_peak = ctx.calibrate()
    rooflines = {}
    for cat, ms in per_proof_ms.items():
        t = ms / 1e3
        if t <= 0:
            continue
        r = {"ms_per_proof": ms}
        if cat in algo:
            a = algo[cat] / t / 1e9
            r["hbm"] = {"achieved": a, "peak": hbm_peak, "unit": "GB/s", "frac": a / hbm_peak,
                        "algorithmic_bytes_per_proof": algo[cat]}
        if cat == "ntt":
            a = work["ntt"] / t / 1e9
            r["int"] = {"achieved": a, "peak": fmul_peak / 1e9, "unit": "G F-mul/s (radix-2 butterflies)",
                        "frac": a / (fmul_peak / 1e9), "butterflies_per_proof": work["ntt"],
                        "alu_pipe_ncu": "57 % (pass A) / 51 % (pass B), issue active 52 % / 46 % "
                                        "(profiles/ntt_pass_2e23.md)"}
        if cat == "update_betas":
            a = work["update_betas"] / t / 1e9
            r["int"] = {"achieved": a, "peak": fmul_peak / 1e9, "unit": "G F-mul/s",
                        "frac": a / (fmul_peak / 1e9), "fmuls_per_proof": work["update_betas"],
                        "alu_pipe_ncu": "54 % in the sparse-rows pass (profiles/update_betas_sparse_2e22.md)"}
        if cat == "merkle":
            r["compressions_per_proof"] = work["merkle_chain"]
            r["note"] = "root and path chains only (latency bound); whole trees: rows.merkle_tree"
        rooflines[cat] = r
    d = rooflines.get(dom, {})
    primary = d.get("int") or d.get("hbm")
    traffic = None
    if dom == "ntt":
        sc = 2.0 ** (logn - 22)
        traffic = sc * (NTT_TRAFFIC_2E22["read"] + NTT_TRAFFIC_2E22["write"])
    roof = {"kernel": dom, "bound": "int" if "int" in d else "hbm", "ms_per_proof": per_proof_ms[dom],
            "traffic": traffic,
            "traffic_note": "DRAM bytes per proof of all transform launches: ncu capture of the n = 2^22 proof "
                            "scaled by n; above the algorithmic bytes by the two-pass intermediate and the first "
                            "pass's twiddle table" if traffic else None}
    if primary:
        roof.update({"achieved": primary["achieved"], "peak": primary["peak"], "unit": primary["unit"],
                     "frac": primary["frac"]})
    if "hbm" in d:
        roof["hbm"] = d["hbm"]
    roof["peak_source"] = {"hbm": peak_src, "int": "gbz_calibrate on this GPU (F_{p^2} multiply chains, "
                                                     "Blake3 compression chains on every SM)"}

    line = {
        "metric": METRIC, "value": value, "unit": "proofs/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 (F_{p^2}, p=2^61-1)",
        "data": "synthetic (SplitMix64 witness)", "config": dict(CONFIG, parallelism="replicas%d" % ws),
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "e2e": {"value": e2e_batch, "unit": "proofs/s", "h2d_bytes_per_step": int(w.nbytes),
                "d2h_bytes_per_step": int(tbytes),
                "api": "gbz_prove_batch, %d slots, the K steps as one call, pinned host buffers" % E2E_LANES,
                "single_call": {"api": "gbz_prove, one synchronised call per step, pinned host buffers",
                                "value": e2e, "p50_ms": 1e3 * float(np.percentile(e2e_lat, 50)),
                                "p99_ms": 1e3 * float(np.percentile(e2e_lat, 99))}},
        "gpu_launches": launches * args.steps,
        "kernel_ms_per_proof": per_proof_ms,
        "roofline": roof,
        "rooflines": rooflines,
        "int_peaks": {"fmul_per_s": fmul_peak, "blake3_per_s": b3_peak},
        "clocks": clk.summary(),
        "transcript_bytes": tbytes,
        "autotune": tuned or None,
    }
    if rank == 0 and not args.no_many:
        line.update(run_rows(gbz, ctx, rt, stream, fmul_peak, b3_peak, hbm_peak))
        line.update(run_many(gbz, O, ctx, repeats=3))
        line.update(run_party_shares(gbz, O, ctx, repeats=3))
        line.update(run_piop(gbz, O, ctx, repeats=3))
        line.update(run_dpcs(gbz, O, ctx, repeats=3))
    if rank == 0:
        # the standalone verifier on this proof's transcript (host code)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            ok, failed = gbz.verify_proof(got.tobytes(), logn, RATE, 1)
            ts.append(time.perf_counter() - t0)
        line["verifier"] = {"api": "gbz_verify_proof (host, one thread)", "ms": 1e3 * min(ts), "accepted": bool(ok),
                            "failed_checks": failed}
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        ref = O.prove(w, logn, RATE, 1, threads=cores)
        dt_cpu = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / dt_cpu, "unit": "proofs/s", "cores": cores, "kind": "port",
                                "sample": "one full proof of the same workload (same witness) on the host"}
        line["transcript_equals_oracle"] = ref == got.tobytes()
    if rank == 0:
        print(json.dumps(line), flush=True)
    gbz.lib.gbz_host_free(hw_p)
    gbz.lib.gbz_host_free(ht_p)
    gbz.lib.gbz_device_free(ctx.h, dw)
    gbz.lib.gbz_device_free(ctx.h, dt)
    ctx.close()


if __name__ == "__main__":
    main()
