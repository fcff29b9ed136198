#!/usr/bin/env python3
"""Generate the golden fixtures in this directory from the reference itself.

Runs oracle/_ref/ref_driver (built from the unmodified reference sources by
oracle/ref/Makefile; x86-64 only) and stores either the full output (small
cases) or the SHA-256 of the exact output bytes (large cases) together with
the parameters that regenerate the inputs.  Run from the repository root:

    make -C oracle/ref && python tests/golden/make_golden.py [section ...]

The fixtures are what pins the CPU restatement in oracle/gbz_oracle.c; the
GPU tests are then checked against that restatement and these fixtures.
"""
import hashlib
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
FULL = os.path.join(ROOT, "oracle", "_ref", "ref_full")
PIGEON = os.path.join(ROOT, "oracle", "_ref", "pigeon_mpi")

# Witness seeds: 0x5EED0000 + workload * 2^16 + instance (1: n = 2^18 at rate 1/4, 2: n = 2^24 at rate 1/2).
SEED_2E18 = 0x5EED0000 + 1 * 65536
SEED_2E24 = 0x5EED0000 + 2 * 65536


def run(*args):
    t = time.time()
    out = subprocess.run([DRIVER, *map(str, args)], check=True, capture_output=True)
    return out.stdout, time.time() - t


def run_full(*args):
    out = subprocess.run([FULL, *map(str, args)], check=True, capture_output=True)
    return out.stdout


def save(name, data):
    with open(os.path.join(HERE, name), "wb") as f:
        f.write(data)


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref")
    # `make_golden.py copcs sumcheck` regenerates only those sections
    only = set(sys.argv[1:])
    if only:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest = json.load(f)
        if "copcs" in only:
            manifest["copcs"] = gen_copcs()
        if "sumcheck" in only:
            manifest["sumcheck"] = gen_sumcheck()
        if "batchopen" in only:
            manifest["batchopen"] = gen_batchopen()
        if "parties" in only:
            manifest["parties"] = gen_parties()
        if "cosumcheck" in only:
            manifest["cosumcheck"] = gen_cosumcheck()
        if "piop" in only:
            manifest["piop"] = gen_piop()
        if "dpcs" in only:
            manifest["dpcs"] = gen_dpcs()
        if "pcspiop" in only:
            manifest["pcspiop"] = gen_pcspiop()
        if "dpcs_timing" in only:
            manifest["dpcs_timing"] = gen_dpcs_timing()
        with open(os.path.join(HERE, "manifest.json"), "w") as f:
            json.dump(manifest, f, indent=1)
        print("updated", sorted(only))
        return
    manifest = {"generator": "tests/golden/make_golden.py", "driver": "oracle/ref/ref_driver.cpp"}

    data, _ = run("field", 200, 11)
    save("field.bin", data)
    manifest["field"] = {"file": "field.bin", "count": 200, "seed": 11}

    data, _ = run("blake3", 64, 12)
    save("blake3.bin", data)
    manifest["blake3"] = {"file": "blake3.bin", "count": 64, "seed": 12}

    data, _ = run("fs", 12, 13)
    save("fs.bin", data)
    manifest["fs"] = {"file": "fs.bin", "count": 12, "seed": 13}

    prng = {}
    for s in (1, 3396, 42, 123457):
        data, _ = run("prng", 24, s)
        save(f"prng_{s}.bin", data)
        prng[str(s)] = {"file": f"prng_{s}.bin", "count": 24}
    manifest["prng"] = prng

    data, _ = run("beta", 6, 14)
    save("beta.bin", data)
    manifest["beta"] = {"file": "beta.bin", "logn": 6, "seed": 14}

    data, _ = run("tensor", 12, 2, 32, 15)
    save("tensor.bin", data)
    manifest["tensor"] = {"file": "tensor.bin", "logn": 12, "logk": 2, "count": 32, "seed": 15}

    data, _ = run("betas", 6, 10, 20, 16, 1)
    save("betas.bin", data)
    manifest["betas"] = {"file": "betas.bin", "logb": 6, "logN": 10, "l": 20, "seed": 16, "prng_seed": 1}

    fft = []
    data, _ = run("fft", 6, 0, 17)
    save("fft_6_fwd.bin", data)
    fft.append({"logn": 6, "inverse": 0, "seed": 17, "file": "fft_6_fwd.bin"})
    data, _ = run("fft", 6, 1, 18)
    save("fft_6_inv.bin", data)
    fft.append({"logn": 6, "inverse": 1, "seed": 18, "file": "fft_6_inv.bin"})
    for logn, inv, seed in [(1, 0, 19), (2, 1, 20), (10, 0, 21), (12, 1, 22), (16, 0, 23), (20, 0, 24)]:
        data, _ = run("fft", logn, inv, seed)
        fft.append({"logn": logn, "inverse": inv, "seed": seed, "sha256": hashlib.sha256(data).hexdigest()})
    for logn, seed in [(14, 25), (18, 26)]:
        data, _ = run("pfft", logn, seed)
        fft.append({"logn": logn, "inverse": 0, "seed": seed, "pfft": 1,
                    "sha256": hashlib.sha256(data).hexdigest()})
    manifest["fft"] = fft

    merkle = []
    data, _ = run("merkle", 5, 27)
    save("merkle_5.bin", data)
    merkle.append({"logN": 5, "seed": 27, "file": "merkle_5.bin"})
    for logN, seed in [(2, 28), (3, 29), (10, 30), (16, 31), (20, 32)]:
        data, _ = run("merkle", logN, seed)
        merkle.append({"logN": logN, "seed": seed, "sha256": hashlib.sha256(data).hexdigest()})
    manifest["merkle"] = merkle

    proofs = []
    data, _ = run("prove", 6, 4, 33, 1, 1)
    save("prove_6_4.bin", data)
    proofs.append({"logn": 6, "rate": 4, "seed": 33, "prng_seed": 1, "file": "prove_6_4.bin"})
    cases = [(5, 2, 34, 1), (7, 2, 35, 1), (8, 4, 36, 7), (10, 2, 37, 1), (11, 4, 38, 99),
             (12, 2, 39, 1), (14, 4, 40, 1), (16, 2, 41, 5),
             (18, 4, SEED_2E18, 1),   # n = 2^18, rate 1/4
             (24, 2, SEED_2E24, 1)]   # n = 2^24, rate 1/2
    for logn, rate, seed, ps in cases:
        data, dt = run("prove", logn, rate, seed, ps, 1)
        proofs.append({"logn": logn, "rate": rate, "seed": seed, "prng_seed": ps, "bytes": len(data),
                       "sha256": hashlib.sha256(data).hexdigest(), "ref_seconds": round(dt, 3)})
        print(f"prove 2^{logn} rate {rate}: {len(data)} B in {dt:.2f} s", flush=True)
    manifest["prove"] = proofs

    manifest["copcs"] = gen_copcs()
    manifest["sumcheck"] = gen_sumcheck()
    manifest["batchopen"] = gen_batchopen()
    manifest["parties"] = gen_parties()
    manifest["cosumcheck"] = gen_cosumcheck()

    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote", os.path.join(HERE, "manifest.json"))


def gen_sumcheck():
    """Sumcheck round forms, one-party distributed sumchecks and the WHIR
    aggregation functions (ref_full)."""
    out = {}
    for name, args in [
        ("zcround_6_0", ("zcround", 6, 0, 71)), ("zcround_8_2", ("zcround", 8, 2, 72)),
        ("bround_6_0", ("bround", 6, 0, 73)), ("bround_7_1", ("bround", 7, 1, 74)),
        ("cubicsc_8_4", ("cubicsc", 8, 4, 75, 1)), ("cubicsc_10_3", ("cubicsc", 10, 3, 76, 9)),
        ("cubicsc_3_4", ("cubicsc", 3, 4, 77, 1)), ("quadsc_8_4", ("quadsc", 8, 4, 78, 1)),
        ("quadsc_11_2", ("quadsc", 11, 2, 79, 5)),
        ("quadsc4_6", ("quadsc4", 6, 95, 1)), ("quadsc4_9", ("quadsc4", 9, 96, 7)),
        ("quadsc4_1", ("quadsc4", 1, 97, 3)),
        ("aggclaims_6_2_3", ("aggclaims", 6, 2, 3, 80, 1)), ("aggclaims_9_4_2", ("aggclaims", 9, 4, 2, 81, 7)),
        ("aggclaims_5_1_1", ("aggclaims", 5, 1, 1, 82, 1)), ("aggarrays_6_3", ("aggarrays", 6, 3, 83)),
        ("aggarrays_8_2", ("aggarrays", 8, 2, 84)), ("aggcommit_8_3_2_4", ("aggcommit", 8, 3, 2, 4, 85, 1)),
        ("aggcommit_10_2_4_8", ("aggcommit", 10, 2, 4, 8, 86, 3)),
        ("aggcommit_7_4_8_4", ("aggcommit", 7, 4, 8, 4, 87, 1)),
        ("tensor_6_8_2_3", ("tensor", 6, 8, 2, 3, 1, 5)), ("tensor_9_16_4_0", ("tensor", 9, 16, 4, 0, 6, 300)),
        ("tensor_4_4_8_1", ("tensor", 4, 4, 8, 1, 0, 0)), ("phase3_6_8_3_2_1", ("phase3", 6, 8, 3, 2, 1, 88)),
        ("phase3_10_16_20_4_5", ("phase3", 10, 16, 20, 4, 5, 89)),
        ("phase3_8_64_7_2_63", ("phase3", 8, 64, 7, 2, 63, 90)),
        ("encconc_8_2_2_4", ("encconc", 8, 2, 2, 4, 91)), ("encconc_10_4_2_16", ("encconc", 10, 4, 2, 16, 92)),
        ("encconc_6_2_4_8", ("encconc", 6, 2, 4, 8, 93)),
    ]:
        save(name + ".bin", run_full(*args))
        out[name] = {"file": name + ".bin", "args": list(args)}
    return out


def gen_copcs():
    """coPCS side (ref_full links every reference translation unit but main.cpp)."""
    copcs = {}
    for name, args in [
        ("multifold5_10_2", ("multifold5", 10, 2, 51)), ("multifold5_12_3", ("multifold5", 12, 3, 52)),
        ("multifold5_9_1", ("multifold5", 9, 1, 53)), ("lagrange_4", ("lagrange", 4, 54)),
        ("lagrange_7", ("lagrange", 7, 55)), ("encode_3_8", ("encode", 3, 8, 4, 6, 56)),
        ("encode_5_6", ("encode", 5, 6, 2, 3, 57)), ("colmerkle_5_8", ("colmerkle", 5, 8, 16, 58)),
        ("colmerkle_2_6", ("colmerkle", 2, 6, 4, 59)), ("colmerkle_32_5", ("colmerkle", 32, 5, 8, 60)),
        ("shares_8_16", ("shares", 8, 16, 61, 0, 1)), ("shares_9_16p", ("shares", 9, 16, 62, 1, 7)),
        ("shares_7_8p", ("shares", 7, 8, 63, 1, 1)), ("aggr_16_24", ("aggr", 16, 24, 64)),
        ("aggr_8_10", ("aggr", 8, 10, 65)), ("aggr_32_6", ("aggr", 32, 6, 66)),
        ("cophase1_10_3", ("cophase1", 10, 3, 67)), ("cophase1_9_2", ("cophase1", 9, 2, 68)),
        ("cophase2_10_3", ("cophase2", 10, 3, 69)), ("cophase2_8_4", ("cophase2", 8, 4, 70)),
    ]:
        data = run_full(*args)
        save(name + ".bin", data)
        copcs[name] = {"file": name + ".bin", "args": list(args)}
    return copcs


def gen_batchopen():
    """Whir_Batch_Open transcripts (ref_full batchopen: the loop of
    Whir.cpp:706-898 on the reference's functions, cross-checked against
    the unmodified Whir_Batch_Open).  Arguments: rate, whir_k, seed, prng
    seed, log2 sizes.  The output ends with the next random() value."""
    out = {}
    for name, args in [
        ("bo_7_5_r16", (16, 4, 101, 1, 7, 5)),
        ("bo_8_8_r8", (8, 4, 102, 3, 8, 8)),
        ("bo_9_7_7_r4", (4, 4, 103, 1, 9, 7, 7)),
        ("bo_10_8_6_r8", (8, 4, 104, 5, 10, 8, 6)),
        ("bo_10_9_r4", (4, 4, 105, 1, 10, 9)),
        ("bo_9_6_r8_k2", (8, 2, 106, 1, 9, 6)),
        ("bo_10_7_r4_k8", (4, 8, 107, 2, 10, 7)),
        ("bo_12_10_10_7_r2", (2, 4, 108, 1, 12, 10, 10, 7)),
        ("bo_13_9_9_9_6_r2", (2, 4, 109, 9, 13, 9, 9, 9, 6)),
        ("bo_16_12_10_r2", (2, 4, 110, 1, 16, 12, 10)),
    ]:
        data = run_full("batchopen", *args)
        e = {"args": list(args), "bytes": len(data), "sha256": hashlib.sha256(data).hexdigest()}
        if name == "bo_7_5_r16":
            save(name + ".bin", data)
            e["file"] = name + ".bin"
        out[name] = e
    return out


# ------------------------------------------------------------ N-party runs
# Per-rank capture records written by oracle/ref/minimpi/capture.cpp: tag,
# count, then count units of these sizes.
CAPTURE_UNIT = {"H2FI": 16, "H2FO": 16, "FRND": 16, "SHRS": 16, "PAGI": 16, "PAGO": 16, "SPDA": 16, "SPDB": 16,
                "SPDC": 16, "WCIA": 16, "FIPK": 16, "GSYI": 16, "GSYO": 16, "GSSG": 16, "SAGI": 16, "SAGO": 16,
                "SFSI": 16, "SFSO": 16, "PMFC": 16, "PEXO": 16, "PEXC": 16, "DBEY": 16, "DBEE": 0,
                "AGCK": 16, "AGCC": 16, "WOPB": 0, "WOPC": 16, "EVLV": 16,
                "GIDX": 4, "RAND": 4, "GSQU": 4, "MTCB": 36, "CTRB": 36, "WCIR": 36}
# the R1CS front end's records (MINIMPI_CAPTURE_PIOP)
CAPTURE_UNIT.update({t: 4 for t in ("RNCT", "PLMN", "SURN", "PCCN", "CBDG", "RDDG", "QDDG", "CBCN", "QDCN")})
CAPTURE_UNIT.update({"DCBL": 36, "DCBR": 36, "SCBA": 16, "SCBB": 16, "SCBC": 16, "DLEY": 16, "DLEE": 0})
CAPTURE_UNIT.update({t: 16 for t in ("DPDL", "DPDR", "DPDO", "DPDW", "GSR0", "GSR1", "GSRK", "SURO", "PCWI", "PCRI",
                                     "PCCD", "PCFS", "CKRO", "CBP1", "CBP2", "CBP3", "CBR1", "CBR2", "CBRR", "CBKK",
                                     "CBCL", "CBIP", "RDIR", "SIP1", "RDRA", "RDRB", "RDRC", "SSVI", "SSVO", "QDP1",
                                     "QDP2", "QDRR", "QDKK", "QDCL", "QDIP", "SIP2", "SIP3")})


def capture_records(path):
    import struct
    b = open(path, "rb").read()
    o, out = 0, []
    while o < len(b):
        tag = b[o:o + 4].decode()
        cnt = struct.unpack_from("<I", b, o + 4)[0]
        o += 8
        n = cnt * CAPTURE_UNIT[tag]
        out.append((tag, cnt, b[o:o + n]))
        o += n
    return out


def expected_open_transcript(ranks, N, logM, rates, npoint=None):
    """The transcript gbz_pcs_open must write (layout: include/gbz.h), rebuilt
    from the reference ranks' own records: every party's round messages
    (PAGI), the leader's aggregates (PAGO) and challenges (H2FO), the roots
    each rank reported, the queries each rank drew (merged party by party,
    as get_segments orders them), the leader's gathered answers and segments
    (GSYO, GSSG), the phase-3 challenges, the final data each party sent
    (SPDA/SPDB/SPDC), and the running claim K, which the reference keeps in a
    local: K0 = F_ip (FIPK), then the updates of coPCS.cpp:1433, 1481-1483,
    1545-1547 on the captured values."""
    import struct
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gbz_oracle as orc
    import gbz_pcs_oracle as po
    sched = po.schedule(N, 1 << logM, rates)
    deg = sched["degrees"]
    fe_list = lambda b: [tuple(int(x) for x in v) for v in np.frombuffer(b, dtype=np.uint64).reshape(-1, 2)]
    rec = lambda tag, count, payload: struct.pack("<II", tag, count) + payload
    lead = ranks[0]
    h2fo = [r[2] for r in lead if r[0] == "H2FO"][logM + 1 if npoint is None else npoint:]
    pago = [r[2] for r in lead if r[0] == "PAGO"]
    pagi = [[r[2] for r in rk if r[0] == "PAGI"] for rk in ranks]
    gidx = [[r for r in rk if r[0] == "GIDX"] for rk in ranks]
    gsyo = [r[2] for r in lead if r[0] == "GSYO"]
    gssg = [r[2] for r in lead if r[0] == "GSSG"]
    K = fe_list([r[2] for r in lead if r[0] == "FIPK"][0])[0]

    def roots_of(kind):
        out = []
        for rk in ranks:
            ctrb = [r[2] for r in rk if r[0] == "CTRB"]
            mt = [r[2] for i, r in enumerate(rk) if r[0] == "MTCB"
                  and struct.unpack_from("<I", r[2])[0] not in (32, 8) and rk[i - 1][0] != "WCIA"]
            out.append(ctrb[1 if rk is not lead else 2][4:] if kind == "batch" else mt[kind][4:])
        return out

    lead_roots = [r[2][4:] for r in lead if r[0] == "CTRB" and struct.unpack_from("<I", r[2])[0] == N]

    def queries(k):
        w = b""
        for rk in range(N):
            words = struct.unpack("<%dI" % gidx[rk][k][1], gidx[rk][k][2])[4:]
            for a, b in zip(words[0::2], words[1::2]):
                w += struct.pack("<II", a, b)
        return w

    out = b""
    out += rec(34, 3 * N, b"".join(pagi[rk][0] for rk in range(N)))
    out += rec(35, 3, pago[0])
    out += rec(36, 1, h2fo[0])
    p = fe_list(pago[0])
    rf = fe_list(h2fo[0])[0]
    K = po.fmul(rf, po.fadd(p[1], po.fmul(rf, p[0])))
    out += rec(41, 1, np.array([K], dtype=np.uint64).tobytes())
    out += rec(32, N, b"".join(roots_of("batch")))
    out += rec(33, 1, lead_roots[1])
    out += rec(37, 2 * sched["queries"][0], queries(0))
    nround = len(rates) - 1
    for i in range(nround):
        d = deg[i + 1]
        out += rec(34, 2 * d * N, b"".join(pagi[rk][1 + i] for rk in range(N)))
        out += rec(35, 2 * d, pago[1 + i])
        c = h2fo[1 + 2 * i]
        s_ = h2fo[2 + 2 * i]
        out += rec(36, 1, c)
        out += rec(32, N, b"".join(roots_of(i)))
        out += rec(33, 1, lead_roots[2 + i])
        out += rec(37, 2 * sched["queries"][i + 1], queries(1 + i))
        out += rec(38, sched["queries"][i + 1], gsyo[i])
        out += rec(39, sched["queries"][i + 1] * d, gssg[i])
        out += rec(40, 1, s_)
        poly = fe_list(pago[1 + i])
        L2 = orc.lagrange_coeff(np.array(fe_list(c)[0], dtype=np.uint64), (2 * d).bit_length() - 1)
        K = (0, 0)
        for k in range(2 * d):
            K = po.fadd(K, po.fmul(poly[k], tuple(int(x) for x in L2[k])))
        if i < nround - 1:
            sv, pk = fe_list(s_)[0], fe_list(s_)[0]
            for y in fe_list(gsyo[i]):
                K = po.fadd(K, po.fmul(pk, y))
                pk = po.fmul(pk, sv)
        out += rec(41, 1, np.array([K], dtype=np.uint64).tobytes())
    fin = b""
    for rk in ranks:
        for tag in ("SPDA", "SPDB", "SPDC"):
            fin += [r[2] for r in rk if r[0] == tag][0]
    out += rec(42, len(fin) // 16, fin)
    return out


def leader_rounds(lead, i):
    """The delegation rounds of the leader's tail from record i (the first
    WHIR commitment of gathered segments): per round the commitment's size
    and root, the extension query draws, prove_multi_folding's and
    prove_extension's claims and the evaluations their checks compute.
    Returns (rounds, the index of the parties' final data)."""
    import struct
    sha = lambda b: hashlib.sha256(b).hexdigest()
    rounds = []
    while True:
        while i < len(lead) and lead[i][0] not in ("WCIA", "SPDA"):
            i += 1
        if lead[i][0] == "SPDA":
            break
        rd = {}
        while lead[i][0] != "WCIR":
            i += 1
        n, = struct.unpack_from("<I", lead[i][2])
        rd["whir_commit"] = n
        rd["root"] = lead[i][2][4:].hex()
        i += 1
        q = []
        while lead[i][0] == "RAND":
            q.append(struct.unpack("<I", lead[i][2])[0])
            i += 1
        rd["queries2"] = q
        ev = []
        while lead[i][0] != "PEXC":
            t, _, p = lead[i]
            if t == "EVLV":
                ev.append(p[16:].hex())
            elif t == "PMFC":
                rd["pmf"] = p.hex()
            elif t == "PEXO":
                rd["pexo_sha256"] = sha(p)
            i += 1
        rd["pex"] = lead[i][2].hex()
        rd["check_evals"] = ev
        rounds.append(rd)
        i += 1
    return rounds, i


def leader_tail(lead):
    """The leader's records after the parties' rounds of PCS_open_new: per
    delegation round the WHIR commitment of the gathered segments, the
    extension query draws, the claims of prove_multi_folding and
    prove_extension with the evaluations their checks compute; then
    aggregate_claims, the openings of aggregate_commitments, _Whir_Open
    (per iteration its commitment root, query draws and the roots of the
    replies it hashes; the final claim) and delegate_beta_eval (its claim and
    the evaluations of its check).  The glibc draws are counted in random()
    calls: forty per F::_random() (two randomNumber() of twenty digits,
    fieldElement.cpp:119-125, 363-368), one per rand()."""
    import struct
    sha = lambda b: hashlib.sha256(b).hexdigest()
    tags = [r[0] for r in lead]
    calls = lambda rs: sum(40 if r[0] == "FRND" else 1 for r in rs if r[0] in ("FRND", "RAND"))
    w0 = tags.index("WCIA")
    # (the calls before the tail are not all seen here: the dealing calls
    # random() directly too; the oracle's restatement of the dealing gives
    # the generator's state where the tail starts)
    out = {"prng_calls": calls(lead[w0:])}
    out["rounds"], i = leader_rounds(lead, w0)
    k = tags.index("AGCK", i)
    out["aggr_K"] = lead[k][2].hex()
    out["aggr_challenges"] = lead[k + 1][2].hex()
    i = k + 2
    q = []
    while lead[i][0] == "RAND":
        q.append(struct.unpack("<I", lead[i][2])[0])
        i += 1
    out["aggr_queries"] = q
    b, e = tags.index("WOPB", i), tags.index("WOPC", i)
    it = []
    j = b
    while j < e:
        if lead[j][0] == "RAND":
            root = lead[j - 1]
            qs = []
            while lead[j][0] == "RAND":
                qs.append(struct.unpack("<I", lead[j][2])[0])
                j += 1
            rr = b"".join(lead[j + t][2][4:] for t in range(len(qs)))
            it.append({"commit": struct.unpack_from("<I", root[2])[0], "root": root[2][4:].hex(), "queries": qs,
                       "reply_roots_sha256": sha(rr)})
            j += len(qs)
        else:
            j += 1
    out["whir_iterations"] = it
    out["whir_evals"] = [lead[t][2][16:].hex() for t in range(b, e) if lead[t][0] == "EVLV"]
    out["whir_claim"] = lead[e][2].hex()
    d = tags.index("DBEY", e)
    out["beta_eval_y"] = lead[d][2].hex()
    de = tags.index("DBEE", d)
    out["beta_eval_evals"] = [lead[t][2][16:].hex() for t in range(d, de) if lead[t][0] == "EVLV"]
    return out


def gen_parties():
    """The reference's own coPCS test (main.cpp:49-163: PCS_commit then
    PCS_open_new) run unmodified with N ranks as N processes (pigeon_mpi,
    minimpi), each rank's transcript captured by link-time interposition.
    Kept per case: what every rank computed that the one-device party
    pipeline must reproduce (full values where small, SHA-256 otherwise)."""
    import struct
    import tempfile
    out = {}
    for N, logM in ((4, 14), (16, 16), (8, 19), (16, 24)):
        with tempfile.TemporaryDirectory() as td:
            prefix = os.path.join(td, "cap")
            env = dict(os.environ, MINIMPI_NP=str(N), MINIMPI_CAPTURE=prefix, MINIMPI_TIMEOUT="300")
            t = time.time()
            log = subprocess.run([PIGEON, "0", str(logM)], env=env, check=True, capture_output=True, text=True)
            dt = time.time() - t
            ranks = [capture_records("%s.%d" % (prefix, r)) for r in range(N)]
        sha = lambda b: hashlib.sha256(b).hexdigest()
        hx = lambda b: b.hex()
        lead = ranks[0]
        npoint = logM + 1
        h2fo = [r[2] for r in lead if r[0] == "H2FO"]
        expected = expected_open_transcript(ranks, N, logM, [[4], [4], [4, 4], [4, 4]])
        case = {"N": N, "logM": logM, "rates": [[4], [4], [4, 4], [4, 4]], "ref_seconds": round(dt, 2),
                "gpu_transcript_bytes": len(expected), "gpu_transcript_sha256": sha(expected),
                "stdout": log.stdout.strip().splitlines(),
                "K": hx([r[2] for r in lead if r[0] == "FIPK"][0]),
                "point_len": npoint,
                "challenges": [hx(x) for x in h2fo[npoint:]],
                "polys": [hx(r[2]) for r in lead if r[0] == "PAGO"],
                "y": [hx(r[2]) for r in lead if r[0] == "GSYO"],
                "segments_sha256": [sha(r[2]) for r in lead if r[0] == "GSSG"],
                "leader": leader_tail(lead),
                "ranks": []}
        small = N * (1 << logM) <= (1 << 20)
        for rk, recs in enumerate(ranks):
            sh = [r[2] for r in recs if r[0] == "SHRS"]
            ctrb = [r[2] for r in recs if r[0] == "CTRB"]
            # commit roots of the opening: MT_commit_Blake calls other than the
            # per-column ones (32 or 8 entries) and the leader's WHIR commitment
            # of the gathered segments (the call right after a WCIA record)
            big_roots = [r[2] for i, r in enumerate(recs) if r[0] == "MTCB"
                         and struct.unpack_from("<I", r[2])[0] not in (32, 8) and recs[i - 1][0] != "WCIA"]
            gidx = []
            for r in recs:
                if r[0] == "GIDX":
                    w = struct.unpack("<%dI" % r[1], r[2])
                    gidx.append(list(w[5::2]))
            e = {"shares_sha256": [sha(x) for x in sh],
                 "base_root": hx(ctrb[0][4:]),
                 "tree_roots": [hx(x[4:]) + ":%d" % struct.unpack_from("<I", x)[0] for x in ctrb],
                 "commit_roots": [hx(x[4:]) + ":%d" % struct.unpack_from("<I", x)[0] for x in big_roots[:3]],
                 "party_polys": [(hx if small else sha)(r[2]) for r in recs if r[0] == "PAGI"],
                 "queries": gidx if small else [sha(str(g).encode()) for g in gidx],
                 "final": [(hx if small else sha)(r[2]) for r in recs if r[0] in ("SPDA", "SPDB", "SPDC")],
                 "final_bytes": [len(r[2]) for r in recs if r[0] in ("SPDA", "SPDB", "SPDC")]}
            case["ranks"].append(e)
        name = "parties_N%d_M%d" % (N, logM)
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(case, f, indent=0)
        out[name] = {"file": name + ".json", "N": N, "logM": logM}
        print("parties N=%d M=2^%d: reference %.1f s" % (N, logM, dt), flush=True)
    return out


COSC = os.path.join(ROOT, "oracle", "_ref", "pigeon_cosc")


def gen_cosumcheck():
    """quadratic_coSumcheck / cubic_coSumcheck run unmodified with N ranks
    (oracle/ref/cosumcheck_mpi_driver.cpp).  Kept: the transcript
    gbz_cosumcheck must write (rebuilt from every rank's captured aggregation
    inputs, the leader's aggregates, challenges and final unpack), the
    leader's claims, and the check flags the reference's messages give."""
    import struct
    import tempfile
    out = {}
    for form, N, logn, degs, seed in (("quad", 4, 10, (8, 4, 4), 21), ("quad", 16, 12, (8, 4, 8), 22),
                                      ("quad", 8, 13, (64, 16), 23), ("cubic", 4, 10, (8, 4, 4), 24),
                                      ("cubic", 16, 12, (16, 8, 4), 25), ("cubic", 8, 11, (4, 4, 4, 4), 26)):
        with tempfile.TemporaryDirectory() as td:
            prefix, res = os.path.join(td, "cap"), os.path.join(td, "claims.bin")
            env = dict(os.environ, MINIMPI_NP=str(N), MINIMPI_CAPTURE=prefix, MINIMPI_TIMEOUT="300")
            log = subprocess.run([COSC, form, str(logn), ",".join(map(str, degs)), str(seed), res], env=env,
                                 check=True, capture_output=True, text=True)
            ranks = [capture_records("%s.%d" % (prefix, r)) for r in range(N)]
            raw = open(res, "rb").read()
        KK, claims = raw[:32], raw[32:]
        rows = 4 if form == "cubic" else 5
        lead = ranks[0]
        h2fo = [r[2] for r in lead if r[0] == "H2FO"]
        sago = [r[2] for r in lead if r[0] == "SAGO"][2:]   # the first two: the driver's claim computation
        sagi = [[r[2] for r in rk if r[0] == "SAGI"][2:] for rk in ranks]
        rec = lambda tag, count, payload: struct.pack("<II", tag, count) + payload
        t = rec(36, 1, h2fo[0])
        for i, d in enumerate(degs):
            D = d * (4 if form == "cubic" else 2)
            t += rec(34, D * N, b"".join(sagi[rk][i] for rk in range(N)))
            t += rec(35, D, sago[i])
            t += rec(36, 1, h2fo[1 + i])
        t += rec(43, rows * N, b"".join([r[2] for r in rk if r[0] == "SFSI"][0] for rk in ranks))
        t += rec(44, rows * (N // 2), [r[2] for r in lead if r[0] == "SFSO"][0])
        t += rec(36, 1, h2fo[-1])
        cnt = struct.unpack_from("<I", claims)[0]
        o, evals = 4, b""
        for _ in range(cnt):
            evals += claims[o:o + 16]
            ln = struct.unpack_from("<I", claims, o + 16)[0]
            o += 20 + 16 * ln
        t += rec(45, cnt, evals)
        msgs = log.stdout
        flags = 0
        for i in range(len(degs)):
            if "ERROR %d\n" % i in msgs:
                flags |= 1 << i
        if "Error in final sumcheck check" in msgs:
            flags |= 1 << 29
        if "Error in final sumcheck verification 2" in msgs:
            flags |= 1 << 30
        name = "cosc_%s_N%d_%d_%s" % (form, N, logn, "_".join(map(str, degs)))
        out[name] = {"form": form, "N": N, "logn": logn, "degrees": list(degs), "seed": seed,
                     "K": KK[:16].hex(), "K_r": KK[16:].hex(), "claims": claims.hex(), "flags": flags, "transcript_bytes": len(t),
                     "transcript_sha256": hashlib.sha256(t).hexdigest(), "stdout": sorted(set(msgs.splitlines()))}
    with open(os.path.join(HERE, "cosumcheck.json"), "w") as f:
        json.dump(out, f, indent=1)
    return {"file": "cosumcheck.json", "cases": sorted(out)}


def gen_piop():
    """The reference's R1CS front end (main.cpp:256-257: coPIOP_prove, pigeon
    1) run unmodified with N ranks, recorded up to the end of its second
    sumcheck (prove_phase1 / prove_phase2, coPIOP.cpp:241-627).  Kept per
    case: where rank 0's generator stood at each dealing step, the digests of
    every rank's dealt inputs (which oracle/gbz_piop_oracle.py regenerates),
    the Fiat-Shamir state the first phase starts from, and what every rank
    computed in the two phases (values where small, SHA-256 otherwise)."""
    import struct
    import tempfile
    out = {}
    for N, logM in ((8, 16), (16, 16), (8, 18), (16, 20)):
        with tempfile.TemporaryDirectory() as td:
            prefix = os.path.join(td, "cap")
            env = dict(os.environ, MINIMPI_NP=str(N), MINIMPI_CAPTURE=prefix, MINIMPI_TIMEOUT="300",
                       MINIMPI_CAPTURE_PIOP="1")
            t = time.time()
            log = subprocess.run([PIGEON, "1", str(logM)], env=env, check=True, capture_output=True, text=True)
            dt = time.time() - t
            ranks = [capture_records("%s.%d" % (prefix, r)) for r in range(N)]
        sha = lambda b: hashlib.sha256(b).hexdigest()
        words = lambda b: list(struct.unpack("<%dI" % (len(b) // 4), b))
        fes = lambda b: [b[i:i + 16].hex() for i in range(0, len(b), 16)]

        def first(recs, tag, after=None):
            i0 = 0 if after is None else next(i for i, r in enumerate(recs) if r[0] == after)
            return next(r[2] for r in recs[i0:] if r[0] == tag)

        def every(recs, tag):
            return [r[2] for r in recs if r[0] == tag]

        lead = ranks[0]
        # the leader's Fiat-Shamir draws from the end of PCS_commit to the end
        # of the second sumcheck
        tags = [r[0] for r in lead]
        i0, i1 = tags.index("PCFS"), tags.index("QDCL")
        draws = [lead[i][2].hex() for i in range(i0, i1) if tags[i] == "H2FO"]
        rn = [words(b) for b in every(lead, "RNCT")]
        plmn = words(first(lead, "PLMN"))
        case = {"N": N, "logM": logM, "rates": [[4], [4], [4, 4], [4, 4]], "ref_seconds": round(dt, 2),
                "logm": plmn[0], "logn": plmn[1], "mask_l": plmn[2],
                "generator": {"seed": rn[0][1], "draws": [[w[0], w[2] + (w[3] << 32)] for w in rn]},
                "pcs_randomness": words(first(lead, "SURN"))[0],
                "degrees1": words(first(lead, "CBDG")), "degrees2": words(first(lead, "QDDG")),
                "K": first(lead, "GSRK").hex(), "fs0": first(lead, "PCFS").hex(),
                "commit_rows": words(first(lead, "PCCN")),
                "draws": draws,
                "phase1": {"r1": fes(first(lead, "CBR1")), "r2": fes(first(lead, "CBR2")),
                           "K_Kr": fes(first(lead, "CBKK")), "Kr": first(lead, "CKRO").hex(),
                           "claims": first(lead, "CBCL").hex(), "claim_points": words(first(lead, "CBCN")),
                           "ip": first(lead, "CBIP").hex()},
                "phase2": {"r": fes(first(lead, "RDIR")), "K_Kr": fes(first(lead, "QDKK")),
                           "claims": first(lead, "QDCL").hex(), "claim_points": words(first(lead, "QDCN")),
                           "ip": first(lead, "QDIP").hex()},
                "errors": [l for l in log.stdout.splitlines() if "ERROR" in l or "Error" in l],
                "ranks": []}
        for recs in ranks:
            suro = every(recs, "SURO")
            e = {"dealt_sha256": {"vL": sha(first(recs, "DPDL")), "vR": sha(first(recs, "DPDR")),
                                  "vO": sha(first(recs, "DPDO")), "W": sha(first(recs, "DPDW")),
                                  "R1": sha(first(recs, "GSR0")), "R2": sha(first(recs, "GSR1")),
                                  "pcs_random": sha(suro[0]), "R": sha(suro[1]),
                                  "commit_data": sha(first(recs, "PCCD"))},
                 "phase1_sha256": {"p1": sha(first(recs, "CBP1")), "p2": sha(first(recs, "CBP2")),
                                   "p3": sha(first(recs, "CBP3")), "ip": sha(first(recs, "SIP1"))},
                 "phase2_sha256": {"RA": sha(first(recs, "RDRA")), "RB": sha(first(recs, "RDRB")),
                                   "RC": sha(first(recs, "RDRC")), "R_aggr": sha(first(recs, "SSVI")),
                                   "reshared": sha(first(recs, "SSVO")), "p1": sha(first(recs, "QDP1")),
                                   "p2": sha(first(recs, "QDP2")),
                                   "ip2": sha(first(recs, "SIP2", after="QDCL")),
                                   "ip3": sha(first(recs, "SIP3", after="QDCL"))}}
            case["ranks"].append(e)
        name = "piop_N%d_M%d" % (N, logM)
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(case, f, indent=0)
        out[name] = {"file": name + ".json", "N": N, "logM": logM}
        print("piop N=%d M=2^%d: reference %.1f s" % (N, logM, dt), flush=True)
    return out


DPCS = os.path.join(ROOT, "oracle", "_ref", "pigeon_dpcs")


def gen_pcspiop():
    """PCS_open_new with isPIOP = true (coPCS.cpp:1310-1700, as coPIOP_prove
    calls it) run unmodified with N ranks after the coPCS test's dealing and
    PCS_commit (oracle/ref/dpcs_mpi_driver.cpp pcs mode: input vectors from
    Lagrange vectors at seeded points, K their F_ip claim).  Kept: the
    transcript gbz_pcs_open_piop's parties' part must equal (rebuilt from
    the ranks' records as for the coPCS test), the leader's delegation rounds,
    r_c, delegate_lagrange_eval's claim and check evaluations, the glibc
    calls of the tail, and the WHIR batch slots 2 and 3 the opening fills."""
    import struct
    import tempfile
    out = {}
    rates = [[4], [4], [4, 4], [4, 4]]
    for N, logM, seed in ((8, 16, 31), (16, 16, 32), (16, 18, 33), (32, 17, 34)):
        with tempfile.TemporaryDirectory() as td:
            prefix, cap = os.path.join(td, "pp"), os.path.join(td, "cap")
            env = dict(os.environ, MINIMPI_NP=str(N), MINIMPI_TIMEOUT="300", MINIMPI_CAPTURE=cap)
            log = subprocess.run([DPCS, "pcs", str(logM), str(seed), prefix], env=env, check=True,
                                 capture_output=True, text=True)
            ranks = [capture_records("%s.%d" % (cap, r)) for r in range(N)]
            b = open(prefix + ".0", "rb").read()
        o = 0
        slots = []
        for _ in range(2):
            sl = {}
            for key in ("arr", "codeword", "betas"):
                (n,) = struct.unpack_from("<I", b, o)
                o += 4
                sl[key + "_sha256"] = hashlib.sha256(b[o:o + 16 * n]).hexdigest()
                sl[key + "_len"] = n
                o += 16 * n
            sl["claim"] = b[o:o + 16].hex()
            sl["root"] = b[o + 16:o + 48].hex()
            o += 48
            slots.append(sl)
        expected = expected_open_transcript(ranks, N, logM, rates, npoint=0)
        lead = ranks[0]
        tags = [t for t, _, _ in lead]
        w0 = tags.index("WCIA")
        rounds, i = leader_rounds(lead, w0)
        d0, d1 = tags.index("DLEY"), tags.index("DLEE")
        calls = lambda rs: sum(40 if r[0] == "FRND" else 1 for r in rs if r[0] in ("FRND", "RAND"))
        case = {"N": N, "logM": logM, "seed": seed, "rates": rates, "K": [p for t, _, p in lead if t == "FIPK"][0].hex(),
                "gpu_transcript_bytes": len(expected), "gpu_transcript_sha256": hashlib.sha256(expected).hexdigest(),
                "stdout": log.stdout.strip().splitlines(),
                "leader": {"rounds": rounds, "prng_calls": calls(lead[w0:]),
                           "r_c": [p for t, _, p in lead[i:d0] if t == "FRND"][0].hex(),
                           "lag_y": lead[d0][2].hex(),
                           "lag_evals": [p[16:].hex() for t, _, p in lead[d0:d1] if t == "EVLV"],
                           "lag_draws": sum(1 for t in tags[d0:d1] if t == "FRND")},
                "whir_slots": slots}
        name = "pcspiop_N%d_M%d" % (N, logM)
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(case, f, indent=0)
        out[name] = {"file": name + ".json", "N": N, "logM": logM}
        print("pcspiop N=%d M=2^%d" % (N, logM), flush=True)
    return out
def gen_dpcs_timing():
    """The reference's own time for the distributed PCS at the benchmark's
    size (bench.py run_dpcs: 16 parties, 2^20 entries each in 16 rows, rate
    4): Batch_dCommit and PIOP_dOpen_batch_new run unmodified with 16 ranks
    on this host's cores (oracle/ref/dpcs_mpi_driver.cpp open mode,
    DPCS_TIMING=1: rank 0's wall time of the first commitment and of the
    opening)."""
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        env = dict(os.environ, MINIMPI_NP="16", MINIMPI_TIMEOUT="1500", DPCS_TIMING="1")
        log = subprocess.run([DPCS, "open", "2", "20", "16", "4", "41", os.path.join(td, "o")], env=env, check=True,
                             capture_output=True, text=True)
    line = [x for x in log.stdout.splitlines() if x.startswith("seconds:")][0].split()
    out = {"N": 16, "logA": 20, "batch": 16, "rate": 4, "P": 2, "commit_seconds": float(line[2]),
           "open_seconds": float(line[4]), "host_cores": os.cpu_count(), "ranks": 16}
    # PCS_open_new with isPIOP at the party-shares size (16 parties, M = 2^24;
    # bench.py run_party_shares' open_piop_ms), the driver's pcs mode
    with tempfile.TemporaryDirectory() as td:
        log = subprocess.run([DPCS, "pcs", "24", "35", os.path.join(td, "p")], env=env, check=True,
                             capture_output=True, text=True)
    line = [x for x in log.stdout.splitlines() if x.startswith("seconds: open_piop")][0].split()
    out["pcs_piop"] = {"N": 16, "logM": 24, "open_seconds": float(line[2])}
    with open(os.path.join(HERE, "dpcs_timing.json"), "w") as f:
        json.dump(out, f, indent=1)
    return {"file": "dpcs_timing.json"}


DPCS_OPEN_CASES = [(2, 8, 12, 8, 4, 21), (2, 16, 13, 8, 4, 22), (3, 8, 11, 4, 2, 23), (2, 32, 11, 4, 4, 24)]
DPCS_CASES = [("batch", 8, 12, 8, 4, 5), ("batch", 16, 14, 16, 4, 6), ("batch", 8, 13, 4, 8, 7),
              ("batch", 32, 10, 32, 2, 8), ("single", 8, 12, 0, 4, 9), ("single", 16, 13, 0, 2, 10),
              ("single", 32, 10, 0, 4, 11)]


def gen_dpcs():
    """Batch_dCommit / dCommit (distributed_PCS.cpp:56-170) run unmodified
    with N ranks (oracle/ref/dpcs_mpi_driver.cpp) on seeded per-rank
    arrays.  Kept per case and rank: the digests of the codeword rows, of
    commit_data (Batch_dCommit) and of every level of the rank's tree, its
    root, and rank 0's leader root."""
    import struct
    import tempfile
    out = {}
    for mode, N, logA, batch, rate, seed in DPCS_CASES:
        A = 1 << logA
        with tempfile.TemporaryDirectory() as td:
            prefix = os.path.join(td, "dp")
            env = dict(os.environ, MINIMPI_NP=str(N), MINIMPI_TIMEOUT="300")
            args = [DPCS, mode, str(logA)] + ([str(batch)] if mode == "batch" else []) + [str(rate), str(seed), prefix]
            subprocess.run(args, env=env, check=True, capture_output=True, text=True)
            ranks = []
            for r in range(N):
                b = open("%s.%d" % (prefix, r), "rb").read()
                o = 0
                if mode == "batch":
                    nb, L = struct.unpack_from("<II", b, 0)
                    o = 8
                    cd = b[o:o + 16 * A]
                    o += 16 * A
                    cw = b[o:o + 16 * nb * L]
                    o += 16 * nb * L
                else:
                    (L,) = struct.unpack_from("<I", b, 0)
                    o = 4
                    cd = None
                    cw = b[o:o + 16 * L]
                    o += 16 * L
                root = b[o:o + 32]
                o += 32
                (cnt,) = struct.unpack_from("<I", b, o)
                o += 4
                lv = b[o:o + 32 * cnt]
                o += 32 * cnt
                e = {"codewords_sha256": hashlib.sha256(cw).hexdigest(), "root": root.hex(),
                     "levels": cnt, "levels_sha256": hashlib.sha256(lv).hexdigest()}
                if cd is not None:
                    e["commit_data_sha256"] = hashlib.sha256(cd).hexdigest()
                if r == 0:
                    e["leader_root"] = b[o:o + 32].hex()
                ranks.append(e)
        name = "%s_N%d_A%d_b%d_r%d" % (mode, N, logA, batch, rate)
        out[name] = {"mode": mode, "N": N, "logA": logA, "batch": batch, "rate": rate, "seed": seed, "ranks": ranks}
    for P, N, logA, batch, rate, seed in DPCS_OPEN_CASES:
        with tempfile.TemporaryDirectory() as td:
            prefix, cap = os.path.join(td, "op"), os.path.join(td, "cap")
            env = dict(os.environ, MINIMPI_NP=str(N), MINIMPI_TIMEOUT="300", MINIMPI_CAPTURE=cap,
                       MINIMPI_CAPTURE_PIOP="1")
            log = subprocess.run([DPCS, "open", str(P), str(logA), str(batch), str(rate), str(seed), prefix], env=env,
                                 check=True, capture_output=True, text=True)
            ranks = [capture_records("%s.%d" % (cap, r)) for r in range(N)]
            b = open(prefix + ".0", "rb").read()
        o = 0

        def fes_at(n):
            nonlocal o
            v = b[o:o + 16 * n]
            o += 16 * n
            return v

        def u32():
            nonlocal o
            (v,) = struct.unpack_from("<I", b, o)
            o += 4
            return v

        y = fes_at(u32())
        polys = fes_at(u32())
        cw = fes_at(u32())
        betas = fes_at(u32())
        claim = fes_at(1)
        root = b[o:o + 32]
        lead = ranks[0]
        tags = [t for t, _, _ in lead]
        hin = [p for t, _, p in lead if t == "H2FI"]
        case = {"mode": "open", "P": P, "N": N, "logA": logA, "batch": batch, "rate": rate, "seed": seed,
                "y": y.hex(), "draws": [p.hex() for t, _, p in lead if t == "H2FO"],
                "eval_claims": hin[0].hex(), "round_polys": [h.hex() for h in hin[4:]],
                "leader_roots": [p[4:].hex() for t, _, p in lead if t == "DCBR"],
                "whir_arr_sha256": hashlib.sha256(polys).hexdigest(), "whir_codeword_sha256": hashlib.sha256(cw).hexdigest(),
                "whir_betas_sha256": hashlib.sha256(betas).hexdigest(), "whir_claim": claim.hex(), "whir_root": root.hex(),
                "gathered_codeword_sha256": hashlib.sha256([p for t, _, p in lead if t == "SCBC"][0]).hexdigest(),
                "errors": [l for l in log.stdout.splitlines() if "Error" in l],
                "ranks": [{"roots": [p[4:].hex() for t, _, p in rk if t == "DCBL"],
                           "queries": [hashlib.sha256(p).hexdigest() for t, _, p in rk if t == "GIDX"]} for rk in ranks]}
        name = "open_P%d_N%d_A%d_b%d_r%d" % (P, N, logA, batch, rate)
        out[name] = case
    with open(os.path.join(HERE, "dpcs.json"), "w") as f:
        json.dump(out, f, indent=1)
    return {"file": "dpcs.json", "cases": sorted(out)}


if __name__ == "__main__":
    main()
