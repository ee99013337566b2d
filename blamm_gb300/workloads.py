"""Seeded synthetic workloads with the shapes of the benchmark cases.

The reference ships no benchmark data; these generators stand in for it:
  two_sequences_1mbp  32 motifs (L 6-20), 2 x 500 kbp iid (A=T=0.3, C=G=0.2)
  genome_100mbp       512 motifs (L 5-30), 24 sequences log-uniform 1-20 Mbp, ~100 Mbp
                      total, iid (A=T=0.29, C=G=0.21)
  genome_1gbp         2000 motifs (L 5-30), 1 Gbp, 2nd-order Markov background
                      (GC ~ 0.41), 1 % of bases in N runs of length log-uniform 100-10k
  promoters_10k       10,000 sequences, log-normal lengths (median 2 kbp, sigma 1.0,
                      clipped 200-50k), GC 0.5, 800 motifs (L 6-25)
  service_*           a resident bank of 2000 motifs (L 5-30); requests of log-uniform
                      length 1 kbp-5 Mbp (iid, GC ~ U[0.35, 0.6]), a subset of
                      U{1..2000} motifs and p in {1e-3, 1e-4, 1e-5}
Motif columns are Multinomial(100, Dirichlet(0.5 * 1_4)) counts.  Random
streams: numpy default_rng with separate children for motifs, lengths, bases.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


def rngs(seed: int) -> tuple[np.random.Generator, np.random.Generator, np.random.Generator]:
    ss = np.random.SeedSequence(seed)
    m, l, b = ss.spawn(3)
    return np.random.default_rng(m), np.random.default_rng(l), np.random.default_rng(b)


def random_pfms(rng: np.random.Generator, nmotifs: int, lmin: int, lmax: int, total: int = 100,
                alpha: float = 0.5) -> list[tuple[str, np.ndarray]]:
    out = []
    for i in range(nmotifs):
        L = int(rng.integers(lmin, lmax + 1))
        probs = rng.dirichlet([alpha] * 4, size=L)
        counts = np.stack([rng.multinomial(total, p) for p in probs]).astype(np.uint64)
        out.append((f"MOTIF{i:05d}", counts))
    return out


def iid_bases(rng: np.random.Generator, n: int, probs) -> np.ndarray:
    idx = rng.choice(4, size=n, p=np.asarray(probs, dtype=np.float64))
    return ACGT[idx]


def markov2_bases(rng: np.random.Generator, n: int, gc: float = 0.41, block: int = 1000) -> np.ndarray:
    """2nd-order Markov chain: seeded 16 x 4 transition table, rows tilted to the GC target.

    Sampled as n / block independent chains of `block` bases advanced together (vectorised
    over the chains); each chain starts from a uniformly drawn two-base context."""
    raw = rng.dirichlet([2.0] * 4, size=16)
    target = np.array([(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2])
    w = target.copy()
    for _ in range(20):  # tilt the rows until the chain's stationary base composition hits the target
        table = raw * w
        table /= table.sum(axis=1, keepdims=True)
        T = np.zeros((16, 16))
        for st in range(16):
            for c in range(4):
                T[st, ((st << 2) | c) & 15] += table[st, c]
        pi = np.full(16, 1 / 16)
        for _ in range(200):
            pi = pi @ T
        comp = np.array([pi[np.arange(16) & 3 == c].sum() for c in range(4)])
        w *= target / comp
    cdf = np.cumsum(table, axis=1)[:, :3]  # symbol = number of cdf entries below u
    nb = (n + block - 1) // block
    state = rng.integers(0, 16, size=nb)
    codes = np.empty((nb, block), dtype=np.uint8)
    for i in range(block):
        u = rng.random(nb)
        c = (u[:, None] >= cdf[state]).sum(axis=1)
        codes[:, i] = c
        state = ((state << 2) | c) & 15
    return ACGT[codes.reshape(-1)[:n]]


def insert_n_runs(rng: np.random.Generator, seq: np.ndarray, frac: float, lmin: int = 100,
                  lmax: int = 10000) -> np.ndarray:
    """Overwrite ~frac of the bases with N runs of log-uniform length."""
    n = len(seq)
    seq = seq.copy()
    budget = int(frac * n)
    while budget > 0:
        L = int(np.exp(rng.uniform(np.log(lmin), np.log(lmax))))
        L = min(L, budget)
        s = int(rng.integers(0, max(1, n - L)))
        seq[s:s + L] = ord("N")
        budget -= L
    return seq


@dataclass
class Workload:
    """FASTA-level description: named sequences (raw bytes, may contain N) + motif PFMs."""
    name: str
    sequences: list[tuple[str, np.ndarray]]
    motifs: list[tuple[str, np.ndarray]]
    pvalue: float = 1e-4
    meta: dict = field(default_factory=dict)

    @property
    def total_bases(self) -> int:
        return int(sum(len(s) for _, s in self.sequences))


def two_sequences_1mbp(seed: int = 0, seq_len: int = 500_000) -> Workload:
    rm, rl, rb = rngs(seed)
    motifs = random_pfms(rm, 32, 6, 20)
    seqs = [(f"seq{i}", iid_bases(rb, seq_len, [0.3, 0.2, 0.2, 0.3])) for i in range(2)]
    return Workload("two_sequences_1mbp", seqs, motifs, 1e-4)


def genome_100mbp(seed: int = 0, total: int = 100_000_000, nseq: int = 24, part: int = 0) -> Workload:
    """part > 0: another `total`-base part of a larger genome (its own sequence lengths and
    bases, the same motifs); part 0 is the workload itself."""
    rm, rl, rb = rngs(seed)
    if part > 0:
        rl, rb = (np.random.default_rng(s) for s in np.random.SeedSequence([seed, part]).spawn(2))
    motifs = random_pfms(rm, 512, 5, 30)
    raw = np.exp(rl.uniform(np.log(1e6), np.log(2e7), size=nseq))
    lens = np.maximum(1, np.round(raw / raw.sum() * total)).astype(np.int64)
    seqs = [(f"chr{part * nseq + i + 1}", iid_bases(rb, int(L), [0.29, 0.21, 0.21, 0.29]))
            for i, L in enumerate(lens)]
    return Workload("genome_100mbp", seqs, motifs, 1e-4, {"lengths": lens.tolist(), "part": part})


def genome_1gbp(seed: int = 0, total: int = 1_000_000_000, nseq: int = 24) -> Workload:
    rm, rl, rb = rngs(seed)
    motifs = random_pfms(rm, 2000, 5, 30)
    raw = np.exp(rl.uniform(np.log(1e6), np.log(2e7), size=nseq))
    lens = np.maximum(1, np.round(raw / raw.sum() * total)).astype(np.int64)
    seqs = []
    for i, L in enumerate(lens):
        s = markov2_bases(rb, int(L), 0.41)
        seqs.append((f"chr{i + 1}", insert_n_runs(rb, s, 0.01)))
    return Workload("genome_1gbp", seqs, motifs, 1e-4, {"lengths": lens.tolist()})


def promoters_10k(seed: int = 0, nseq: int = 10_000) -> Workload:
    rm, rl, rb = rngs(seed)
    motifs = random_pfms(rm, 800, 6, 25)
    lens = np.clip(np.round(np.exp(rl.normal(np.log(2000), 1.0, size=nseq))), 200, 50_000).astype(np.int64)
    seqs = [(f"prom{i}", iid_bases(rb, int(L), [0.25, 0.25, 0.25, 0.25])) for i, L in enumerate(lens)]
    return Workload("promoters_10k", seqs, motifs, 1e-4, {"lengths": lens.tolist()})


def service_bank(seed: int = 0) -> list[tuple[str, np.ndarray]]:
    rm, _, _ = rngs(seed)
    return random_pfms(rm, 2000, 5, 30)


SERVICE_PVALUES = (1e-3, 1e-4, 1e-5)


def service_requests(seed: int, k: int, nmotifs: int = 2000, max_len: int = 5_000_000):
    """k serving requests: (bases, run starts [0], motif indices (sorted), p-value index)."""
    rng = np.random.default_rng([seed, 5])
    out = []
    for _ in range(k):
        n = int(np.exp(rng.uniform(np.log(1_000), np.log(max_len))))
        gc = rng.uniform(0.35, 0.6)
        b = iid_bases(rng, n, [(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2])
        m = int(rng.integers(1, nmotifs + 1))
        motifs = np.sort(rng.choice(nmotifs, size=m, replace=False))
        out.append((b, np.zeros(1, dtype=np.int64), motifs, int(rng.integers(0, len(SERVICE_PVALUES)))))
    return out


# ---------------------------------------------------------------- writers
def write_fasta(path: str, sequences: list[tuple[str, np.ndarray]], width: int = 60) -> None:
    with open(path, "wb") as f:
        for name, seq in sequences:
            f.write(b">" + name.encode() + b"\n")
            b = seq.tobytes()
            for i in range(0, len(b), width):
                f.write(b[i:i + width] + b"\n")


def write_jaspar(path: str, motifs: list[tuple[str, np.ndarray]]) -> None:
    with open(path, "w") as f:
        for name, pfm in motifs:
            f.write(f">{name}\t{name}\n")
            for k, ch in enumerate("ACGT"):
                f.write(ch + "  [ " + " ".join(f"{int(v):5d}" for v in pfm[:, k]) + " ]\n")


def write_cb(path: str, motifs: list[tuple[str, np.ndarray]]) -> None:
    with open(path, "w") as f:
        for name, pfm in motifs:
            f.write(f">{name}\n")
            for row in pfm:
                f.write("\t".join(str(int(v)) for v in row) + "\n")


def write_settings(path: str, w: int = 250, h: int = 1000, tile_area: int = 4096,
                   pseudo: float = 0.25, flush: int = 100000) -> None:
    with open(path, "w") as f:
        f.write(f"MATRIX_S_W\t{w}\nMATRIX_S_H\t{h}\nMATRIX_P_TILE_MIN_ZERO_AREA\t{tile_area}\n"
                f"PSEUDOCOUNT\t{pseudo}\nFLUSHOUTPUT\t{flush}\n")


def write_case(directory: str, groups: dict[str, list[tuple[str, list[tuple[str, np.ndarray]]]]],
               motifs: list[tuple[str, np.ndarray]], jaspar: bool = True) -> tuple[str, str]:
    """groups: {group: [(fasta_file_name, sequences), ...]} -> (motif_file, manifest)."""
    os.makedirs(directory, exist_ok=True)
    lines = []
    for g, files in groups.items():
        for fname, seqs in files:
            write_fasta(os.path.join(directory, fname), seqs)
            lines.append(f"{g}\t{fname}\n")
    manifest = os.path.join(directory, "sequences.mf")
    with open(manifest, "w") as f:
        f.writelines(lines)
    mfile = os.path.join(directory, "motifs.jaspar" if jaspar else "motifs.cb")
    (write_jaspar if jaspar else write_cb)(mfile, motifs)
    return mfile, manifest


# ---------------------------------------------------------------- streams
def filtered_stream(sequences: list[tuple[str, np.ndarray]]):
    """FASTA content -> (bases, run_start, run_seq, run_seqpos): maximal runs of ACGTacgt.

    Same stream the host library builds from FASTA files (one line per
    sequence, so line breaks never split a run)."""
    valid = np.zeros(256, dtype=bool)
    valid[np.frombuffer(b"ACGTacgt", dtype=np.uint8)] = True
    parts, starts, rseq, rpos = [], [], [], []
    n = 0
    for si, (_, seq) in enumerate(sequences):
        v = valid[seq]
        if not v.any():
            continue
        d = np.diff(np.concatenate([[0], v.view(np.int8), [0]]))
        b = np.flatnonzero(d == 1)
        e = np.flatnonzero(d == -1)
        for s0, e0 in zip(b, e):
            starts.append(n)
            rseq.append(si)
            rpos.append(int(s0))
            parts.append(seq[s0:e0])
            n += int(e0 - s0)
    bases = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint8)
    return (bases, np.asarray(starts, dtype=np.int64), np.asarray(rseq, dtype=np.int64),
            np.asarray(rpos, dtype=np.int64))
