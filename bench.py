#!/usr/bin/env python
"""Benchmark of the GB300 PWM scan: bp*motif/s on the 512-motif x 100 Mbp workload.

One step = one scan of the whole synthetic stream (both strands, p = 1e-4
thresholds from theoretical histograms) through libblamm_gpu's C ABI:
  value : device-resident stream and hit buffer (blamm_scan_device), CUDA events
          on the library's stream around every step, L2 flushed between steps
  e2e   : host buffers (blamm_scan): H2D of the stream and run table, the scan,
          D2H of the hits, wall clock per step
The headline mode is the BF16 hi+lo split on tcgen05; the single-term BF16 and
the plain FP32 GPU forms run on the same stream and must give the same hits.
`--impl reference` times the reference's own CPU algorithm (the oracle's port of
its BLAS loop; the reference binary cannot be built on the GPU host) instead.

Prints one JSON line (rank 0).  Multi-GPU (torchrun): each rank scans its own
contiguous share of the sequences, no collective on the data path.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bp·motif/s on 1 GB300, BF16-split vs FP32 plain (same hits); serve p50/p99 ms"
UNIT = "bp·motif/s"


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--bases", type=int, default=100_000_000, help="total bases of the workload")
    ap.add_argument("--cpu-sample", type=int, default=8_000_000, help="bases in a CPU-baseline sample")
    ap.add_argument("--no-modes", action="store_true", help="skip the bf16 / fp32 comparison runs")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-cli", action="store_true", help="skip the end-to-end command-line measurement")
    ap.add_argument("--mode", default="auto", choices=["auto", "bf16", "bf16x2", "e4m3"],
                    help="headline arithmetic: auto (the library default, autotuned on a sample) or a fixed "
                         "term count with the default tile plan (no autotuner launches, for profiling)")
    ap.add_argument("--serve-requests", type=int, default=48, help="distinct requests of the serving pool")
    ap.add_argument("--serve-slots", type=int, default=8, help="requests in flight in the serving measurement")
    ap.add_argument("--workload", default="genome_100mbp", choices=["genome_100mbp", "genome_1gbp", "promoters_10k"],
                    help="genome_100mbp is the headline line; genome_1gbp (1 Gbp x 2000 motifs, precision at scale) and "
                         "promoters_10k (10,000 short sequences, batching) print their own measurement line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------ workload
def _genome(seed: int, total: int, part: int, genome_counts):
    from blamm_gb300 import workloads  # numpy generators only: no native library is loaded
    wl = workloads.genome_100mbp(seed, total=total, part=part)
    bases, runs, rseq, _ = workloads.filtered_stream(wl.sequences)
    counts = np.array([np.count_nonzero((bases | 0x20) == ord(c)) for c in "acgt"], dtype=np.uint64)
    if genome_counts is not None:
        counts = genome_counts(counts)
    return wl, bases, runs, rseq, counts


def build_workload(seed: int, total: int, part: int = 0, genome_counts=None):
    """genome_100mbp (part 0) or another part of the same genome through the product's host
    library (motif bank, PWMs, p-value thresholds); genome_counts maps this part's A/C/G/T
    counts to the whole genome's (the PWM background of every part).  Also returns, per P
    column, the index of its PFM in the workload's motif list and its strand (1 = reverse)."""
    from blamm_gb300._native import MotifBank
    wl, bases, runs, rseq, counts = _genome(seed, total, part, genome_counts)
    bank = MotifBank.from_pfms([p for _, p in wl.motifs], revcompl=True)
    bank.generate(counts, 0.25)
    P, lens, rc = bank.matrix()
    tot = np.float32(counts.sum()) + np.float32(4.0) * np.float32(0.25)
    bgp = ((counts.astype(np.float32) + np.float32(0.25)) / tot).astype(np.float32)
    thr = bank.pvalue_thresholds(bgp, wl.pvalue)
    colmotif = np.array([int(bank.name(c)[1:]) for c in range(P.shape[0])], dtype=np.int64)
    return wl, bases, runs, rseq, P, lens, thr, (colmotif, rc.astype(np.int8))


def build_workload_oracle(seed: int, total: int):
    """The same workload set up by the oracle alone (the reference's PWM, matrix and threshold
    steps restated in C): the reference arm loads nothing of the product."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    wl, bases, runs, rseq, counts = _genome(seed, total, 0, None)
    P, lens, thr, colmotif, strand = oracle.motif_bank([p for _, p in wl.motifs], counts, 0.25, (wl.pvalue,))
    return wl, bases, runs, rseq, P, lens, thr[0], (colmotif, strand)


def sample_digest(h: np.ndarray, colkey) -> dict:
    """Order-independent digest of a hit set keyed by (position, PFM index, strand, score bits),
    so that two differently ordered banks of the same motifs compare."""
    colmotif, strand = colkey
    if len(h) == 0:
        return {"hits": 0, "digest": 0}
    key = ((h["pos"].astype(np.uint64) << np.uint64(24)) ^ (colmotif[h["col"]].astype(np.uint64) << np.uint64(1))
           ^ strand[h["col"]].astype(np.uint64)) * np.uint64(0x9E3779B97F4A7C15)
    key ^= h["score"].view(np.uint32).astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)
    return {"hits": int(len(h)), "digest": int(np.bitwise_xor.reduce(key))}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names[1:], parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), "measured (MEASURED_PEAKS.json bf16_tflops, burst)"
    return 1900.0, "fallback 1.9 PFLOP/s"


def profile_traffic(positions: int, terms: int):
    """DRAM bytes of one scan-kernel launch (the instance for `terms` BF16 terms) over
    `positions` positions, scaled by positions from the committed ncu capture."""
    path = os.path.join(ROOT, "profiles", "scan_tc_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    c = d["by_terms"].get(str(terms))
    return None if c is None else int(c["dram_bytes"] * positions / c["positions"])


def hit_digest(h: np.ndarray) -> tuple[int, int]:
    """Order-independent digest of a hit set (count, checksum of pos/col/score bits)."""
    key = (h["pos"].astype(np.uint64) * np.uint64(1_000_003) + h["col"].astype(np.uint64)) ^ (
        h["score"].view(np.uint32).astype(np.uint64) << np.uint64(20))
    return int(len(h)), int(np.bitwise_xor.reduce(key * np.uint64(0x9E3779B97F4A7C15)) if len(h) else 0)


# ------------------------------------------------------------------ CPU side
def cpu_sample_scan(bases, runs, P, lens, thr, sample: int, threads: int | None = None):
    """The reference's BLAS loop (oracle port) on the first `sample` bases, all cores
    (or `threads` workers, the reference's -t).  Returns (rate, cores, seconds, hits): the
    hits of every window that ends inside the sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    b = bases[:sample]
    r = runs[runs < len(b)]
    tiles = oracle.matrix_tiles(lens, 4096)
    cores = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    h = oracle.scan_blas(b, r, P, lens, thr, tiles, 1000, 250, cores)
    dt = time.perf_counter() - t0
    return len(b) * P.shape[0] / dt, cores, dt, h


def restrict_to_sample(h: np.ndarray, lens, sample: int) -> np.ndarray:
    """Hits of a whole-stream scan whose window ends inside the first `sample` bases."""
    return h[h["pos"] + lens[h["col"]] <= sample]


def parity_vs_oracle(gpu_hits: np.ndarray, oracle_hits: np.ndarray, lens, sample: int) -> dict:
    """Bit-for-bit comparison on the sample: the same (position, column) set and the same
    score bits."""
    a = np.sort(restrict_to_sample(gpu_hits, lens, sample), order=["pos", "col"])
    b = np.sort(oracle_hits, order=["pos", "col"])
    same = (len(a) == len(b) and np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["col"], b["col"])
            and np.array_equal(a["score"].view(np.uint32), b["score"].view(np.uint32)))
    return {"positions": int(sample), "hits": int(len(b)), "gpu_hits": int(len(a)), "identical": bool(same)}


def product_libraries_loaded() -> list[str]:
    """This process's mapped shared libraries that belong to the product (blamm_gb300/)."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")}
    except OSError:
        return ["unknown: /proc/self/maps unreadable"]
    pkg = os.path.realpath(os.path.join(ROOT, "blamm_gb300"))
    return sorted(p for p in paths if os.path.realpath(p).startswith(pkg))


def cli_e2e(wl, bases, sample: int) -> dict:
    """The reference's command line on the CPU sample, end to end: FASTA in, occurrence file
    out, `scan -rc -pt 1e-4 -t <cores>` through the oracle's port of the reference's CLI on its
    BLAS block loop (OpenBLAS, one BLAS thread per worker).  `dict` is written directly (the
    sample's sequences with the whole genome's base counts, so that the PWMs are the headline's)
    and `hist` runs untimed beforehand, as the reference's own workflow runs them once."""
    import shutil
    import subprocess
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from blamm_gb300 import workloads
    blas = oracle.find_blas()
    if not os.path.exists(oracle.CLI_PATH) or not blas:
        return {"unavailable": "oracle CLI or an LP64 BLAS missing"}
    d = tempfile.mkdtemp(prefix="blamm_cli_")
    try:
        seqs, left = [], sample
        for name, s in wl.sequences:
            if left <= 0:
                break
            seqs.append((name, s[:left]))
            left -= len(s[:left])
        workloads.write_fasta(os.path.join(d, "sample.fa"), seqs)
        with open(os.path.join(d, "sequences.mf"), "w") as f:
            f.write("genome\tsample.fa\n")
        workloads.write_jaspar(os.path.join(d, "motifs.jaspar"), wl.motifs)
        workloads.write_settings(os.path.join(d, "settings.cnf"))
        counts = [int(np.count_nonzero((bases | 0x20) == ord(c))) for c in "acgt"]
        with open(os.path.join(d, "sequences.mf.dict"), "w") as f:
            f.write(f"NUM_SPECIES\t1\nSPECIES\tgenome\nNUM_FASTA_FILES\t1\nsample.fa\n"
                    f"TOT_SEQ_LENGTH\t{sample}\nNUCL_COUNT_ACGT\t" + "\t".join(map(str, counts)) +
                    f"\nNUM_SEQUENCES\t{len(seqs)}\n" + "".join(n + "\n" for n, _ in seqs))
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1", BLAMM_ORACLE_BLAS=blas)
        subprocess.run([oracle.CLI_PATH, "hist", "motifs.jaspar", "sequences.mf"], cwd=d, env=env, check=True,
                       stdout=subprocess.DEVNULL)
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        subprocess.run([oracle.CLI_PATH, "scan", "-rc", "-pt", str(wl.pvalue), "-t", str(cores), "motifs.jaspar",
                        "sequences.mf"], cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
        dt = time.perf_counter() - t0
        with open(os.path.join(d, "occurrences.txt"), "rb") as f:
            lines = sum(1 for _ in f)
        return {"value": sample * 2 * len(wl.motifs) / dt, "unit": UNIT, "seconds": dt, "cores": cores,
                "occurrence_lines": lines,
                "sample": f"first {sample} bp (FASTA, {len(seqs)} sequences) x {2 * len(wl.motifs)} columns: "
                          "read, scan, write the occurrence file"}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def cli_ours(wl, pvalue: float) -> dict:
    """The drop-in command line on the whole workload, end to end: the FASTA files of the
    genome, `blamm dict` (timed), `blamm hist` (untimed, run once as the workflow does) and
    `blamm scan -rc -pt <p>` (timed) writing the occurrence file; the scan's phase split
    (BLAMM_TIMING) with the default GPU FASTA reader, and the scan's time with the host
    reader beside it."""
    import re
    import shutil
    import subprocess
    import tempfile
    from blamm_gb300 import workloads
    from blamm_gb300._native import CLI_PATH
    d = tempfile.mkdtemp(prefix="blamm_cli_ours_")
    try:
        workloads.write_case(d, {"genome": [("genome.fa", wl.sequences)]}, wl.motifs)
        workloads.write_settings(os.path.join(d, "settings.cnf"))
        out = {}

        def run(args, env=None):
            t0 = time.perf_counter()
            r = subprocess.run([CLI_PATH] + args, cwd=d, capture_output=True, text=True,
                               env=dict(os.environ, **(env or {})))
            dt = time.perf_counter() - t0
            if r.returncode != 0:
                raise RuntimeError(f"blamm {args[0]} failed: {r.stderr[-500:]}")
            return dt, r.stderr

        out["dict_seconds"], _ = run(["dict", "sequences.mf"])
        out["dict_seconds_host_reader"], _ = run(["dict", "sequences.mf"], {"BLAMM_FASTA_READER": "host"})
        run(["hist", "motifs.jaspar", "sequences.mf"])
        scan = ["scan", "-rc", "-pt", str(pvalue), "motifs.jaspar", "sequences.mf"]
        run(scan)  # warm: page cache, GPU context
        out["scan_seconds"], err = run(scan, {"BLAMM_TIMING": "1"})
        m = re.search(r"timing: (.*)", err)
        out["scan_phases"] = m.group(1).strip() if m else None
        with open(os.path.join(d, "occurrences.txt"), "rb") as f:
            out["occurrence_lines"] = sum(1 for _ in f)
        out["occurrence_bytes"] = os.path.getsize(os.path.join(d, "occurrences.txt"))
        out["scan_seconds_host_reader"], err = run(scan, {"BLAMM_FASTA_READER": "host", "BLAMM_TIMING": "1"})
        m = re.search(r"timing: (.*)", err)
        out["scan_phases_host_reader"] = m.group(1).strip() if m else None
        bp = sum(len(s) for _, s in wl.sequences)
        out["value"] = bp * 2 * len(wl.motifs) / out["scan_seconds"]
        out["unit"] = UNIT
        out["workload"] = (f"{bp} bp FASTA ({len(wl.sequences)} sequences, 60-base lines) x "
                           f"{2 * len(wl.motifs)} columns -> occurrence file")
        return out
    except Exception as e:  # reported, not fatal to the bench line
        return {"unavailable": str(e)[:300]}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def run_reference(a, rank, world):
    """--impl reference: the reference's CPU scan (oracle port of its BLAS loop) per step."""
    if rank != 0:
        return
    wl, bases, runs, rseq, P, lens, thr, colkey = build_workload_oracle(a.seed, a.bases)
    sample = min(a.cpu_sample, len(bases))
    for _ in range(a.warmup):
        cpu_sample_scan(bases, runs, P, lens, thr, sample)
    vals, times = [], []
    cores, hits = 1, None
    for _ in range(a.steps):
        v, cores, dt, hits = cpu_sample_scan(bases, runs, P, lens, thr, sample)
        vals.append(v)
        times.append(dt)
    value = float(np.mean(vals))
    cli = cli_e2e(wl, bases, sample)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic",
        "config": {"workload": f"genome_100mbp: 512 motifs (1024 columns, L 5-30, both strands) x "
                               f"{len(bases)} bp, p=1e-4; each step a {sample} bp sample"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
                         "sample": f"first {sample} bp of the stream x 1024 columns, "
                                   "the reference's BLAS block loop (h=1000, w=250) on OpenBLAS"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        # the sample's hits keyed by (position, PFM, strand, score bits): the GPU arm prints the
        # same digest of its headline hits restricted to the sample
        "sample_hits": sample_digest(hits, colkey) if hits is not None else None,
        "cli_e2e": cli,
        "setup": "motif bank, PWMs and p-value thresholds from the oracle",
        "product_libraries_loaded": product_libraries_loaded(),
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ precision of the MMA scores
def fp64_window_scores(bases, P, lens, npos: int) -> np.ndarray:
    """FP64 sum of the FP32 PWM entries for positions [0, npos) x every column (uppercase bases)."""
    code = np.full(len(bases) + 512, 4, dtype=np.int64)
    for v, ch in enumerate(b"ACGT"):
        code[:len(bases)][bases == ch] = v
    ncols = P.shape[0]
    ref = np.zeros((npos, ncols), dtype=np.float64)
    Pz = np.concatenate([P.astype(np.float64), np.zeros((ncols, 4))], axis=1)
    zero = P.shape[1]
    for c in range(ncols):
        for j in range(int(lens[c])):
            b = code[j:j + npos]
            ref[:, c] += Pz[c, np.where(b < 4, 4 * j + b, zero)]
    return ref


def mma_score_error(sc, bases, P, lens, ref, npos: int = 2048) -> dict:
    """Raw tensor-core scores (sum of the fixed-point BF16 terms, before rescoring) of the first
    npos positions x every column, against the FP64 sum of the FP32 PWM entries."""
    bases = bases[:npos + 256]
    raw = sc.debug_scores(bases, 0, npos).astype(np.float64)
    valid = (np.arange(npos)[:, None] + lens[None, :]) <= len(bases)
    err = np.abs(raw - ref)[valid]
    rel = (np.abs(raw - ref) / np.maximum(np.abs(ref), 1.0))[valid]
    return {"positions": npos, "columns": int(P.shape[0]), "max_abs": float(err.max()),
            "mean_abs": float(err.mean()), "max_rel": float(rel.max()), "rel_denominator": "max(|fp64 score|, 1)"}


def emitted_score_error(hits, ref, npos: int) -> dict:
    """Emitted hit scores (FP32, rescored) of positions < npos against the FP64 sums."""
    h = hits[hits["pos"] < npos]
    f64 = ref[h["pos"], h["col"]]
    rel = np.abs(h["score"].astype(np.float64) - f64) / np.maximum(np.abs(f64), 1e-30)
    return {"hits": int(len(h)), "max_rel": float(rel.max()) if len(h) else 0.0,
            "note": "the reference's own FP32 sum; error = FP32 rounding of the sequential sum"}


def precision_other_configs(seed: int, npos: int = 2048) -> dict:
    """Score error against FP64 on the other cases' shapes, each on a sample generated like the
    case itself: the raw tensor-core sums (one and two BF16 terms, one E4M3 term) and the emitted
    scores."""
    from blamm_gb300 import GpuScanner, workloads
    from blamm_gb300._native import MotifBank
    rng = np.random.default_rng([seed, 9])
    cases = {}
    w1 = workloads.two_sequences_1mbp(seed, seq_len=npos + 512)
    cases["two_sequences_1mbp (32 motifs, L 6-20, iid A=T=0.3)"] = (w1.motifs, w1.sequences[0][1], 1e-4)
    m3 = workloads.random_pfms(rng, 2000, 5, 30)
    s3 = workloads.insert_n_runs(rng, workloads.markov2_bases(rng, 200_000, 0.41), 0.01)
    b3, r3, _, _ = workloads.filtered_stream([("s", s3)])
    cases["genome_1gbp (2000 motifs, L 5-30, 2nd-order Markov GC 0.41, N runs), p=1e-5"] = (m3, b3, 1e-5)
    m4 = workloads.random_pfms(rng, 800, 6, 25)
    cases["promoters_10k (800 motifs, L 6-25, GC 0.5)"] = (m4, workloads.iid_bases(rng, npos + 512, [0.25] * 4), 1e-4)
    out = {}
    for name, (motifs, bases, pv) in cases.items():
        bases = np.ascontiguousarray(bases[:npos + 512])
        counts = np.array([max(1, np.count_nonzero((bases | 0x20) == ord(c))) for c in "acgt"], dtype=np.uint64)
        bank = MotifBank.from_pfms([p for _, p in motifs], revcompl=True)
        bank.generate(counts, 0.25)
        P, lens, _ = bank.matrix()
        bgp = ((counts.astype(np.float32) + np.float32(0.25)) /
               (np.float32(counts.sum()) + np.float32(1.0))).astype(np.float32)
        thr = bank.pvalue_thresholds(bgp, pv)
        ref = fp64_window_scores(bases, P, lens, npos)
        res = {}
        for mode in ("bf16x2", "bf16", "e4m3"):
            sc = GpuScanner(0, mode)
            sc.set_motifs(P, lens, thr)
            res["mma_" + mode] = mma_score_error(sc, bases, P, lens, ref, npos)
            if mode == "bf16x2":
                res["emitted"] = emitted_score_error(sc.scan(bases, np.zeros(1, dtype=np.int64)), ref, npos)
            sc.close()
        out[name] = res
    return out


# ------------------------------------------------------------------ serving
def run_serve(a) -> dict:
    """Serving through the scan service (include/blamm_serve.h): a resident bank of
    2000 motifs (4000 columns) with threshold sets for p = 1e-3, 1e-4, 1e-5; requests of
    log-uniform 1 kbp-5 Mbp, U{1..2000} motifs, a random p.  First the saturation throughput
    (every request queued at once), then Poisson arrivals at 25 / 50 / 90 % of it; latency =
    submission to completion, measured by the service."""
    from blamm_gb300 import Server, workloads
    from blamm_gb300._native import MotifBank
    pfms = workloads.service_bank(a.seed)
    bank = MotifBank.from_pfms([p for _, p in pfms], revcompl=True)
    counts = np.array([2625, 2375, 2375, 2625], dtype=np.uint64)  # GC 0.475, the middle of the requests' range
    bank.generate(counts, 0.25)
    P, lens, _ = bank.matrix()
    bgp = ((counts.astype(np.float32) + np.float32(0.25)) /
           (np.float32(counts.sum()) + np.float32(1.0))).astype(np.float32)
    sets = np.stack([bank.pvalue_thresholds(bgp, pv) for pv in workloads.SERVICE_PVALUES])
    reqs = workloads.service_requests(a.seed, a.serve_requests)
    req_cols = [np.stack([2 * m, 2 * m + 1], axis=1).ravel().astype(np.int32) for _, _, m, _ in reqs]
    work = [len(b) * len(c) for (b, _, _, _), c in zip(reqs, req_cols)]
    srv = Server(P, lens, sets, slots=a.serve_slots)
    try:
        for i in range(min(len(reqs), a.serve_slots)):  # warm-up: contexts, buffers, plans
            srv.wait(srv.submit(reqs[i][0][:20_000], reqs[i][1], req_cols[i], reqs[i][3]))
        # saturation: the whole pool queued at once
        t0 = time.perf_counter()
        ids = [srv.submit(b, r, c, st) for (b, r, _, st), c in zip(reqs, req_cols)]
        lat = [srv.wait(i)[1] for i in ids]
        wall = time.perf_counter() - t0
        for i in ids:
            srv.take(i)
        sat_rate = len(reqs) / wall
        out = {"workload": "service: 2000 motifs (4000 columns), requests log-uniform 1 kbp-5 Mbp, "
                           "U{1..2000} motifs, p in {1e-3, 1e-4, 1e-5}",
               "slots": a.serve_slots, "pool": len(reqs),
               "saturation": {"requests_per_s": sat_rate, "bp_motif_per_s": sum(work) / wall,
                              "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))},
               "open_loop": []}
        rng = np.random.default_rng(a.seed + 77)
        for load in (0.25, 0.5, 0.9):
            rate = load * sat_rate
            nreq = int(min(3 * len(reqs), max(len(reqs), rate * 6.0)))
            gaps = rng.exponential(1.0 / rate, size=nreq)
            order = rng.integers(0, len(reqs), size=nreq)
            ids = []
            t0 = time.perf_counter()
            t_next = t0
            for g, k in zip(gaps, order):
                t_next += g
                d = t_next - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                b, r, _, st = reqs[k]
                ids.append(srv.submit(b, r, req_cols[k], st))
            res = [srv.wait(i) for i in ids]
            wall = time.perf_counter() - t0
            for i in ids:
                srv.take(i)
            lat = [x[1] for x in res]
            out["open_loop"].append({"load": load, "rate_req_s": rate, "requests": nreq,
                                     "p50_ms": float(np.percentile(lat, 50)),
                                     "p99_ms": float(np.percentile(lat, 99)),
                                     "bp_motif_per_s": float(sum(work[k] for k in order)) / wall})
        return out
    finally:
        srv.close()


# ------------------------------------------------------------------ configs 3 and 4
def _bank_for(pfms, counts, pvalues, sc):
    """Bank (rc interleaved) + thresholds per p-value from GPU theoretical histograms."""
    from blamm_gb300._native import MotifBank
    bank = MotifBank.from_pfms([p for _, p in pfms], revcompl=True)
    bank.generate(counts, 0.25)
    P, lens, _ = bank.matrix()
    bgp = ((counts.astype(np.float32) + np.float32(0.25)) /
           (np.float32(counts.sum()) + np.float32(1.0))).astype(np.float32)
    t0 = time.perf_counter()
    thr, _ = sc.theoretical_hist(P, lens, bgp, pvalues, hist_of=bank.hist_columns())
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    host = bank.pvalue_thresholds(bgp, pvalues[0])
    t_host = time.perf_counter() - t0
    same = bool(np.array_equal(host.view(np.uint32), thr[0].view(np.uint32)))
    return P, lens, thr, {"gpu_s_all_pvalues": t_gpu, "host_s_one_pvalue": t_host, "gpu_equals_host": same}


def _device_scan(sc, torch, d_b, n, d_r, nr, cap):
    from blamm_gb300 import HIT_DTYPE
    d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), nr, d_h.data_ptr(), cap)
    return nh, d_h


def run_genome_1gbp(a):
    """2000 motifs (4000 columns) over 1 Gbp (2nd-order Markov, GC 0.41, 1 % N runs),
    p = 1e-4 and 1e-5 thresholds inverted in FP64 on the GPU; BF16 split vs single-term BF16
    vs one E4M3 term (same hits required); the plain FP32 form on a 100 Mbp sample."""
    import torch
    from blamm_gb300 import GpuScanner, HIT_DTYPE, workloads
    t0 = time.perf_counter()
    wl = workloads.genome_1gbp(a.seed, total=a.bases if a.bases != 100_000_000 else 1_000_000_000)
    bases, runs, _, _ = workloads.filtered_stream(wl.sequences)
    gen_s = time.perf_counter() - t0
    counts = np.array([np.count_nonzero((bases | 0x20) == ord(c)) for c in "acgt"], dtype=np.uint64)
    sc = GpuScanner(0, "bf16x2")
    P, lens, thr, tinfo = _bank_for(wl.motifs, counts, (1e-4, 1e-5), sc)
    n, ncols = len(bases), P.shape[0]
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    out = {"workload": f"genome_1gbp: 2000 motifs (4000 columns) x {n} bp (2nd-order Markov, GC 0.41, 1% N runs), "
                       "thresholds from GPU theoretical histograms (FP64 inversion)",
           "generate_s": gen_s, "thresholds": tinfo, "runs": []}
    for pi, pv in enumerate((1e-4, 1e-5)):
        sc.set_motifs(P, lens, thr[pi])
        res = {"pvalue": pv}
        digests = {}
        for mode in ("bf16x2", "bf16", "e4m3"):
            sc.set_mode(mode)
            from blamm_gb300 import HIT_DTYPE as HD
            nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), 0, 0, overflow_ok=True)
            cap = nh + 1024
            d_h = torch.empty(cap * HD.itemsize, dtype=torch.uint8, device="cuda")
            ts = []
            for _ in range(3):
                nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
                ts.append(sc.stats())
            st = ts[-1]
            h = d_h[: nh * HD.itemsize].cpu().numpy().view(HD)
            digests[mode] = hit_digest(h)
            if mode == "bf16x2":
                # parity on a sample of this workload: the oracle's scan of the first bases
                # (Markov background, N runs) against the GPU hits of the windows inside them
                sys.path.insert(0, os.path.join(ROOT, "oracle"))
                import oracle
                smp = min(n, a.cpu_sample // 4)
                oh = oracle.scan(bases[:smp], runs[runs < smp], P, lens, thr[pi], nthreads=os.cpu_count() or 8)
                res["parity_vs_oracle"] = parity_vs_oracle(h, oh, lens, smp)
            kern = float(np.median([t["scan_ms"] for t in ts]))
            tot = float(np.median([t["kernel_ms"] for t in ts]))
            res[mode] = {"hits": int(nh), "candidates": int(st["candidates"]), "scan_kernel_ms": kern,
                         "all_kernels_ms": tot, "bp_motif_per_s": n * ncols / (tot / 1e3),
                         "tiles": int(st["tiles"])}
            del d_h
        res["same_hits_bf16_vs_bf16x2"] = digests["bf16"] == digests["bf16x2"]
        res["same_hits_e4m3_vs_bf16x2"] = digests["e4m3"] == digests["bf16x2"]
        out["runs"].append(res)
    # plain FP32 form on a 100 Mbp sample of the same stream, same hits as the split there
    m = min(n, 100_000_000)
    rs = runs[runs < m]
    sc.set_motifs(P, lens, thr[0])
    sample = {}
    for mode in ("fp32", "bf16x2"):
        sc.set_mode(mode)
        from blamm_gb300 import HIT_DTYPE as HD
        d_rs = torch.from_numpy(rs).cuda()
        cap = sc.scan_device(d_b.data_ptr(), m, d_rs.data_ptr(), len(rs), 0, 0, overflow_ok=True) + 1024
        d_h = torch.empty(cap * HD.itemsize, dtype=torch.uint8, device="cuda")
        nh = sc.scan_device(d_b.data_ptr(), m, d_rs.data_ptr(), len(rs), d_h.data_ptr(), cap)
        st = sc.stats()
        sample[mode] = {"hits": int(nh), "kernel_ms": float(st["kernel_ms"]),
                        "bp_motif_per_s": m * ncols / (st["kernel_ms"] / 1e3),
                        "digest": hit_digest(d_h[: nh * HD.itemsize].cpu().numpy().view(HD))}
        del d_h
    sample["same_hits"] = sample["fp32"].pop("digest") == sample["bf16x2"].pop("digest")
    sample["bases"] = m
    out["fp32_sample_p1e-4"] = sample
    sc.close()
    print(json.dumps({"metric": METRIC, "config": out}), flush=True)


def run_promoters_10k(a):
    """10,000 promoter-like sequences (log-normal lengths, median 2 kbp, sigma 1.0,
    clipped 200 bp-50 kbp, GC 0.5) x 800 motifs (1600 columns), p = 1e-4: one persistent launch
    over all sequences, the same as a CUDA graph, and one launch per sequence, in the default mode
    (one BF16 term until tuned); then the autotuned term count and plan."""
    import torch
    from blamm_gb300 import GpuScanner, HIT_DTYPE, workloads
    wl = workloads.promoters_10k(a.seed)
    bases, runs, rseq, _ = workloads.filtered_stream(wl.sequences)
    counts = np.array([np.count_nonzero((bases | 0x20) == ord(c)) for c in "acgt"], dtype=np.uint64)
    sc = GpuScanner(0, "auto")
    P, lens, thr, _ = _bank_for(wl.motifs, counts, (1e-4,), sc)
    sc.set_motifs(P, lens, thr[0])
    n, ncols = len(bases), P.shape[0]
    units = n * ncols
    d_b = torch.from_numpy(bases).cuda()
    d_r = torch.from_numpy(runs).cuda()
    cap = max(1 << 20, units // 1000)
    d_h = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    ext = torch.cuda.ExternalStream(sc.stream())

    def timed(fn, reps=5):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            fn()
            e1.record(ext)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    one = timed(lambda: sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap))
    nh = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
    batch = hit_digest(d_h[: nh * HIT_DTYPE.itemsize].cpu().numpy().view(HIT_DTYPE))
    # a CUDA graph of the enqueued scan
    sc.reserve(n, cap)
    d_c = torch.zeros(4, dtype=torch.int64, device="cuda")
    g = sc.graph_create(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap, d_c.data_ptr())
    graph_ms = timed(lambda: sc.graph_launch(g))
    sc.graph_destroy(g)
    # one launch per sequence (host loop, synchronous calls), on a share of the sequences
    seq_start = np.concatenate([[0], np.cumsum([len(s) for _, s in wl.sequences])])
    k = min(len(wl.sequences), 2000)
    d_one = torch.zeros(1, dtype=torch.int64, device="cuda")
    t0 = time.perf_counter()
    per_hits = 0
    for i in range(k):
        a0, a1 = int(seq_start[i]), int(seq_start[i + 1])
        per_hits += sc.scan_device(d_b.data_ptr() + a0, a1 - a0, d_one.data_ptr(), 1, d_h.data_ptr(), cap)
    torch.cuda.synchronize()
    per_seq_ms = (time.perf_counter() - t0) * 1e3 * len(wl.sequences) / k
    # the autotuned plan
    best = sc.autotune(d_b.data_ptr(), n, d_r.data_ptr(), len(runs))
    tuned = timed(lambda: sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap))
    nh2 = sc.scan_device(d_b.data_ptr(), n, d_r.data_ptr(), len(runs), d_h.data_ptr(), cap)
    same = hit_digest(d_h[: nh2 * HIT_DTYPE.itemsize].cpu().numpy().view(HIT_DTYPE)) == batch
    out = {"workload": f"promoters_10k: {len(wl.sequences)} sequences ({n} bp) x 800 motifs (1600 columns), p=1e-4",
           "one_launch_ms": one, "one_launch_bp_motif_per_s": units / (one / 1e3),
           "graph_ms": graph_ms, "graph_bp_motif_per_s": units / (graph_ms / 1e3),
           "per_sequence_launches_ms": per_seq_ms, "per_sequence_bp_motif_per_s": units / (per_seq_ms / 1e3),
           "per_sequence_sample": f"first {k} sequences, extrapolated to all",
           "autotuned_ms": tuned, "autotune_plan": list(sc.plan_options()), "autotune_terms": sc.terms(),
           "autotuned_same_hits": same,
           "hits": int(nh)}
    sc.close()
    print(json.dumps({"metric": METRIC, "config": out}), flush=True)


# ------------------------------------------------------------------ GPU side
def run_ours(a, rank, world, local):
    import torch
    from blamm_gb300 import GpuScanner, HIT_DTYPE
    from blamm_gb300._native import gpu_lib
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    if world > 1:
        # weak scaling: rank r scans part r of a genome of world x --bases bases (its own
        # sequences, the same motif bank); the PWM background is the whole genome's base
        # composition, summed over the ranks once before any timing (no data-path collective)
        def genome_counts(c):
            t = torch.from_numpy(c.astype(np.int64)).to(f"cuda:{local}")
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
            return t.cpu().numpy().astype(np.uint64)
        wl, bases, runs, rseq, P, lens, thr, colkey = build_workload(a.seed, a.bases, rank, genome_counts)
    else:
        wl, bases, runs, rseq, P, lens, thr, colkey = build_workload(a.seed, a.bases)
    n, ncols = len(bases), P.shape[0]
    units = n * ncols
    flops_per_bp = float(8 * lens.astype(np.int64).sum())

    sc = GpuScanner(local, a.mode)
    sc.set_motifs(P, lens, thr)
    ext = torch.cuda.ExternalStream(sc.stream())
    d_bases = torch.from_numpy(bases).to(f"cuda:{local}")
    d_runs = torch.from_numpy(runs).to(f"cuda:{local}")
    # the library's default mode picks one or two BF16 terms (and the tile plan) from timed
    # scans of a 16 Mi-position sample of the stream; untimed, as a deployment would do once
    tuned_ms = sc.autotune(d_bases.data_ptr(), n, d_runs.data_ptr(), len(runs)) if a.mode == "auto" else None
    terms = sc.terms()
    tuned = {"terms": terms, "max_tile_columns": sc.plan_options()[0], "job_cost": sc.plan_options()[1],
             "sample_kernel_ms": tuned_ms}
    cap = max(1 << 20, units // 2000)
    d_hits = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{local}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def device_steps(k: int, record: bool):
        ms, scan_ms, launches, nh = [], [], 0, 0
        for i in range(k):
            flush.fill_(i & 0xFF)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            nh = sc.scan_device(d_bases.data_ptr(), n, d_runs.data_ptr(), len(runs), d_hits.data_ptr(), cap)
            e1.record(ext)
            e1.synchronize()
            st = sc.stats()
            if record:
                ms.append(e0.elapsed_time(e1))
                scan_ms.append(st["scan_ms"])
                launches += st["launches"]
        return ms, scan_ms, launches, nh

    def hits_on_device(nh: int) -> np.ndarray:
        return d_hits[: nh * HIT_DTYPE.itemsize].cpu().numpy().view(HIT_DTYPE)

    # ---- headline: the default (autotuned) mode
    device_steps(max(a.warmup, 3), False)
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ms, scan_ms, launches, nh = device_steps(a.steps, True)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    step_ms = float(np.sum(ms)) / a.steps
    if dist:
        t = torch.tensor([step_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
        u = torch.tensor([float(units)], device=f"cuda:{local}")
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        total_units = float(u.item())
    else:
        total_units = float(units)
    value = total_units / (step_ms / 1e3)
    st = sc.stats()
    headline_hits = hits_on_device(nh)
    ref_digest = hit_digest(headline_hits)

    # ---- the same step end to end through host buffers (pinned)
    lib = gpu_lib()
    hb = torch.from_numpy(bases).pin_memory()
    hr = torch.from_numpy(runs).pin_memory()
    hh = torch.empty(cap * HIT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    nhc = C.c_int64(0)

    def e2e_step():
        rc = lib.blamm_scan(sc.h, C.c_void_p(hb.data_ptr()), n, C.c_void_p(hr.data_ptr()), len(runs),
                            C.c_void_p(hh.data_ptr()), cap, C.byref(nhc))
        if rc != 0:
            raise RuntimeError(lib.blamm_last_error(sc.h).decode())
    for _ in range(max(a.warmup, 3)):
        e2e_step()
    e2e_t = []
    for _ in range(a.steps):
        t1 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t1)
    e2e_st = sc.stats()
    e2e_digest = hit_digest(hh[: nhc.value * HIT_DTYPE.itemsize].numpy().view(HIT_DTYPE))
    # median over the steps: a single host-side stall (seen now and then on the pinned copies)
    # would otherwise dominate the mean of a few steps; the mean and the maximum are reported too
    e2e_med = float(np.median(e2e_t))
    if dist:  # the slowest rank's median step
        t = torch.tensor([e2e_med], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_med = float(t.item())
    e2e_value = total_units / e2e_med

    # ---- other modes on the same stream (same hits required)
    modes = {}
    if not a.no_modes:
        # each fixed form with the library's default tile plan (the autotuned knobs suit the
        # headline's term count)
        keep_plan = sc.plan_options()
        sc.set_plan_options(256, 700.0)
        for mode in ("bf16x2", "bf16", "e4m3", "fp32"):
            sc.set_mode(mode)
            device_steps(1, False)
            mms, msc, _, mnh = device_steps(max(1, min(3, a.steps)), True)
            mst = sc.stats()
            modes[mode] = {"value": units / (float(np.mean(mms)) / 1e3), "ms_per_step": float(np.mean(mms)),
                           "scan_kernel_ms": float(np.mean(msc)), "hits": int(mnh),
                           "candidates": int(mst["candidates"]),
                           "same_hits_as_headline": hit_digest(hits_on_device(mnh)) == ref_digest}
        sc.set_mode(a.mode)
        sc.set_plan_options(*keep_plan)

    # ---- score error of the tensor-core sums against FP64 (emitted scores are rescored in FP32)
    precision = {}
    if rank == 0:
        npos = 2048
        ref = fp64_window_scores(bases[:npos + 256], P, lens, npos)
        for mode in ("bf16x2", "bf16", "e4m3"):
            sc.set_mode(mode)
            precision["mma_" + mode] = mma_score_error(sc, bases, P, lens, ref, npos)
        sc.set_mode(a.mode)
        precision["emitted"] = emitted_score_error(hits_on_device(nh), ref, npos)
        precision["other_cases"] = precision_other_configs(a.seed)

    # ---- roofline of the dominant kernel (tcgen05 scan)
    peak, peak_src = peaks()
    kern_ms = float(np.mean(scan_ms))
    achieved = n * flops_per_bp / (kern_ms / 1e3) / 1e12
    # a step = packing + (one-hot entries + scan) per scan window + rescoring
    scan_launches = max(1, (launches // a.steps - 2) // 2)
    traffic = profile_traffic(int(round(n / scan_launches)), terms)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ({2: "bf16x2 (hi+lo fixed-point split", 8: "e4m3 (one E4M3 term of P x 2^k"}
                  .get(terms, "bf16 (one fixed-point term"))
                 + ", fp32 accumulate) + fp32 rescoring"
                 + ("; form autotuned" if a.mode == "auto" else ""),
        "data": "synthetic (seeded numpy; the 100 Mbp x 512-motif shapes)",
        "config": {"workload": "genome_100mbp: 512 motifs (1024 columns, L 5-30, both strands, Dirichlet(0.5) "
                               "columns of 100 counts) x 24 iid sequences (A=T=0.29) log-uniform 1-20 Mbp, "
                               f"{n} bp per rank, p=1e-4 theoretical-histogram thresholds",
                   "bases_per_rank": n, "columns": ncols, "l2": "flushed (256 MiB write between steps)",
                   "parallelism": f"{world} rank(s), each its own {n} bp part of the genome, no collective",
                   "autotuned": tuned},
        # the same rate counting a motif's forward and reverse-strand columns once
        "value_per_distinct_motif": value * len(wl.motifs) / ncols,
        "hits": int(nh), "candidates": int(st["candidates"]), "tiles": int(st["tiles"]),
        "scan_kernel_ms": kern_ms, "rescore_kernel_ms": float(st["rescore_ms"]),
        "wall_s_timed_region": wall,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(n + 8 * len(runs)),
                "d2h_bytes_per_step": int(16 * nhc.value + 8), "ms_per_step": 1e3 * e2e_med,
                "stat": f"median of {len(e2e_t)} calls", "ms_per_step_mean": 1e3 * float(np.mean(e2e_t)),
                "ms_per_step_max": 1e3 * float(np.max(e2e_t)),
                "call_kernel_ms": float(e2e_st["kernel_ms"]), "call_total_ms": float(e2e_st["total_ms"]),
                "same_hits": e2e_digest == ref_digest},
        "gpu_launches": int(launches),
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "scan_launches_per_step": scan_launches,
                     "note": f"algorithmic flops = 8 * sum(L) = {flops_per_bp:.0f} per bp over {n} bp in "
                             f"{scan_launches} window launch(es) per step, divided by their summed time; "
                             f"traffic per launch ({n / scan_launches:.0f} positions); "
                             + (f"{terms} BF16 term(s) issue {terms} MMA(s) per flop (ceiling {1 / terms:g} "
                                if terms in (1, 2) else "one E4M3 term: half the BF16 MMA instructions per flop "
                                "at twice the BF16 rate (ceiling 2 of the BF16 peak ")
                             + f"before padding and the bias MMA); peak {peak_src}"},
        "modes": modes,
        "score_error_vs_fp64": precision,
        "clocks": clk,
    }
    if rank == 0 and world == 1 and not a.no_serve:
        sc.close()
        line["serve"] = run_serve(a)
        if line["serve"]["open_loop"]:
            line["serve_p50_ms"] = line["serve"]["open_loop"][-1]["p50_ms"]
            line["serve_p99_ms"] = line["serve"]["open_loop"][-1]["p99_ms"]
    if rank == 0 and world == 1 and not a.no_cli and a.workload == "genome_100mbp":
        line["cli"] = cli_ours(wl, wl.pvalue)
    if rank == 0 and world == 1:
        v, cores, dt, ohits = cpu_sample_scan(bases, runs, P, lens, thr, min(a.cpu_sample, n))
        # parity on the headline workload: the GPU headline hits of every window inside the sample
        # against the oracle's port of the reference's BLAS loop, bit for bit
        smp = min(a.cpu_sample, n)
        line["parity_vs_oracle"] = parity_vs_oracle(headline_hits, ohits, lens, smp)
        line["sample_hits"] = sample_digest(restrict_to_sample(headline_hits, lens, smp), colkey)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
                                "sample": f"first {min(a.cpu_sample, n)} bp x {ncols} columns in {dt:.1f} s: the "
                                          "reference's BLAS block loop (h=1000, w=250, OpenBLAS sgemm per tile "
                                          "per offset, one BLAS thread per worker)"}
        # the reference's -t 1 on a sixteenth of that sample (a few seconds of one core)
        s1 = max(1, min(a.cpu_sample // 16, n))
        v1, _, dt1, _ = cpu_sample_scan(bases, runs, P, lens, thr, s1, threads=1)
        line["cpu_baseline"]["one_thread"] = {"value": v1, "unit": UNIT,
                                              "sample": f"first {s1} bp x {ncols} columns in {dt1:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    sc.close()
    if dist:
        dist.destroy_process_group()


def main():
    a = args_parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    if a.workload == "genome_1gbp":
        if rank == 0:
            run_genome_1gbp(a)
        return
    if a.workload == "promoters_10k":
        if rank == 0:
            run_promoters_10k(a)
        return
    run_ours(a, rank, world, local)


if __name__ == "__main__":
    main()
