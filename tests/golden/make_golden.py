#!/usr/bin/env python
"""Generates the golden fixtures: seeded synthetic inputs + the reference's outputs.

Each case directory holds the inputs (FASTA files, manifest, motif file,
settings.cnf) and, under expected/, what the compiled reference
(oracle/_ref/blamm, built from the reference sources by oracle/build_ref.sh)
wrote for the commands listed in case.json: the .dict, hist_*.dat/.gnu,
PWMthresholds.txt and the occurrence files (sorted; the reference's line order
depends on its thread schedule).

Run in the development container, where the reference sources exist:
    python tests/golden/make_golden.py
The GPU host never runs this; it only reads the committed results.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from blamm_gb300 import workloads  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "blamm")


def seq_with_features(rng, n, probs, n_frac=0.0, lower_frac=0.0, iupac=False):
    s = workloads.iid_bases(rng, n, probs)
    if n_frac:
        s = workloads.insert_n_runs(rng, s, n_frac, 5, 200)
    if lower_frac:
        for _ in range(max(1, int(lower_frac * n / 40))):
            a = int(rng.integers(0, n))
            s[a:a + int(rng.integers(1, 80))] |= 0x20
    if iupac:
        for _ in range(max(1, n // 5000)):
            s[int(rng.integers(0, n))] = ord("RYKMSWBDHV"[int(rng.integers(0, 10))])
    return s


def write_fasta(path, seqs, width=60, crlf=False, empty_line=False):
    nl = b"\r\n" if crlf else b"\n"
    with open(path, "wb") as f:
        for name, s in seqs:
            f.write(b">" + name.encode() + b" some description" + nl)
            b = s.tobytes()
            for i in range(0, len(b), width):
                f.write(b[i:i + width] + nl)
            if empty_line:
                f.write(nl)


def case_mixed(d):
    """Two groups, three files, N runs, lowercase, IUPAC codes, CRLF, an empty sequence,
    a permutation motif (name__1), JASPAR format."""
    rng = np.random.default_rng(101)
    g1a = [(f"g1a_s{i}", seq_with_features(rng, int(rng.integers(2000, 30000)), [0.3, 0.2, 0.2, 0.3],
                                           n_frac=0.01, lower_frac=0.05, iupac=True)) for i in range(6)]
    g1a.insert(3, ("g1a_empty", np.zeros(0, dtype=np.uint8)))
    g1b = [(f"g1b_s{i}", seq_with_features(rng, int(rng.integers(1000, 20000)), [0.25] * 4,
                                           n_frac=0.02)) for i in range(5)]
    g2 = [(f"g2_s{i}", seq_with_features(rng, int(rng.integers(5000, 40000)), [0.2, 0.3, 0.3, 0.2],
                                         lower_frac=0.02)) for i in range(4)]
    os.makedirs(os.path.join(d, "seqs"), exist_ok=True)
    write_fasta(os.path.join(d, "seqs", "b_file.fa"), g1a, width=60, empty_line=True)
    write_fasta(os.path.join(d, "seqs", "a_file.fa"), g1b, width=70, crlf=True)
    write_fasta(os.path.join(d, "seqs", "c_file.fa"), g2, width=80)
    with open(os.path.join(d, "sequences.mf"), "w") as f:
        f.write("group1\tseqs/b_file.fa\ngroup2\tseqs/c_file.fa\ngroup1\tseqs/a_file.fa\n")
    motifs = workloads.random_pfms(rng, 10, 5, 24)
    perm = (motifs[2][0] + "__1", motifs[2][1][rng.permutation(motifs[2][1].shape[0])])
    motifs.append(perm)
    workloads.write_jaspar(os.path.join(d, "motifs.jaspar"), motifs)
    workloads.write_settings(os.path.join(d, "settings.cnf"))
    return {"motifs": "motifs.jaspar", "manifest": "sequences.mf",
            "commands": [["dict", "sequences.mf"],
                         ["hist", "motifs.jaspar", "sequences.mf"],
                         ["scan", "-rc", "-pt", "0.0001", "-o", "occ_pt.txt", "motifs.jaspar", "sequences.mf"],
                         ["scan", "-rt", "0.9", "-o", "occ_rt.txt", "motifs.jaspar", "sequences.mf"],
                         ["scan", "-rc", "-at", "8", "-o", "occ_at.txt", "motifs.jaspar", "sequences.mf"],
                         ["scan", "-s", "-rc", "-rt", "0.92", "-o", "occ_simple.txt", "motifs.jaspar",
                          "sequences.mf"]],
            "outputs": ["occ_pt.txt", "occ_rt.txt", "occ_at.txt", "occ_simple.txt"]}


def case_cb(d):
    """Cluster-Buster motifs, forward strand only, a small hist (-b 100 -l 200000)."""
    rng = np.random.default_rng(202)
    seqs = [(f"chr{i}", seq_with_features(rng, 40000, [0.3, 0.2, 0.2, 0.3], n_frac=0.005)) for i in range(3)]
    os.makedirs(os.path.join(d, "seqs"), exist_ok=True)
    write_fasta(os.path.join(d, "seqs", "genome.fa"), seqs)
    with open(os.path.join(d, "sequences.mf"), "w") as f:
        f.write("sp\tseqs/genome.fa\n")
    motifs = workloads.random_pfms(rng, 8, 6, 18)
    workloads.write_cb(os.path.join(d, "motifs.cb"), motifs)
    workloads.write_settings(os.path.join(d, "settings.cnf"), pseudo=0.5)
    return {"motifs": "motifs.cb", "manifest": "sequences.mf",
            "commands": [["dict", "sequences.mf"],
                         ["hist", "-b", "100", "-l", "200000", "motifs.cb", "sequences.mf"],
                         ["scan", "-pt", "0.001", "-o", "occ_pt.txt", "motifs.cb", "sequences.mf"],
                         ["scan", "-rc", "-rt", "0.88", "-o", "occ_rt.txt", "motifs.cb", "sequences.mf"]],
            "outputs": ["occ_pt.txt", "occ_rt.txt"]}


def case_two_sequences_1mbp(d):
    """The two-sequence case at full size: 32 motifs (L 6-20), 2 x 500 kbp iid (A=T=0.3), -rc -pt 1e-4.
    The FASTA file and the occurrence file are stored gzip-compressed (see COMPRESS)."""
    wl = workloads.two_sequences_1mbp(0, seq_len=500_000)
    os.makedirs(os.path.join(d, "seqs"), exist_ok=True)
    workloads.write_fasta(os.path.join(d, "seqs", "seqs.fa"), wl.sequences)
    with open(os.path.join(d, "sequences.mf"), "w") as f:
        f.write("cfg1\tseqs/seqs.fa\n")
    workloads.write_jaspar(os.path.join(d, "motifs.jaspar"), wl.motifs)
    workloads.write_settings(os.path.join(d, "settings.cnf"))
    return {"motifs": "motifs.jaspar", "manifest": "sequences.mf",
            "commands": [["dict", "sequences.mf"],
                         ["hist", "motifs.jaspar", "sequences.mf"],
                         ["scan", "-rc", "-pt", "0.0001", "-o", "occ_pt.txt", "motifs.jaspar", "sequences.mf"],
                         ["hist", "-e", "-l", "150000", "-H", "emp", "motifs.jaspar", "sequences.mf"]],
            "outputs": ["occ_pt.txt"]}


CASES = {"mixed": case_mixed, "cb": case_cb, "two_sequences_1mbp": case_two_sequences_1mbp}

# files kept gzip-compressed in the fixtures (tests/golden_cases.py inflates them)
COMPRESS = {"two_sequences_1mbp": ["seqs/seqs.fa", "expected/occ_pt.txt"]}


def compress(d, files):
    import gzip
    for f in files:
        p = os.path.join(d, f)
        with open(p, "rb") as fi, gzip.GzipFile(p + ".gz", "wb", compresslevel=9, mtime=0) as fo:
            shutil.copyfileobj(fi, fo)
        os.remove(p)


def run_reference(d, spec):
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    os.makedirs(os.path.join(d, "emp"), exist_ok=True)
    for cmd in spec["commands"]:
        args = [REF] + cmd
        if cmd[0] == "scan" or (cmd[0] == "hist" and "-e" in cmd):
            args = [REF, cmd[0], "-t", "4"] + cmd[1:]
        res = subprocess.run(args, cwd=d, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
        if res.returncode != 0:
            raise RuntimeError(f"reference failed: {args}\n{res.stderr.decode()}")


def collect(d, spec):
    exp = os.path.join(d, "expected")
    if os.path.exists(exp):
        shutil.rmtree(exp)
    os.makedirs(exp)
    for f in sorted(os.listdir(d)):
        p = os.path.join(d, f)
        if f.endswith(".dict") or f.startswith("hist_") or f == "PWMthresholds.txt":
            shutil.move(p, os.path.join(exp, f))
        elif f in spec["outputs"]:
            with open(p, "rb") as fh:
                lines = sorted(fh.read().splitlines(keepends=True))
            with open(os.path.join(exp, f), "wb") as fh:
                fh.writelines(lines)
            os.remove(p)
    emp = os.path.join(d, "emp")
    if os.path.isdir(emp):
        if os.listdir(emp):
            shutil.move(emp, os.path.join(exp, "emp"))
        else:
            os.rmdir(emp)


def main():
    if not os.path.exists(REF):
        sys.exit("build the reference first: oracle/build_ref.sh")
    for name, fn in CASES.items():
        d = os.path.join(HERE, name)
        if os.path.exists(d):
            shutil.rmtree(d)
        os.makedirs(d)
        spec = fn(d)
        run_reference(d, spec)
        collect(d, spec)
        compress(d, COMPRESS.get(name, []))
        with open(os.path.join(d, "case.json"), "w") as f:
            json.dump(spec, f, indent=1)
        print(name, "ok")


if __name__ == "__main__":
    main()
