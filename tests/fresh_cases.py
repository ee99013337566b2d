"""Fresh inputs for differential tests: a case directory (FASTA files, manifest, motifs,
settings.cnf) and the `blamm` commands to run in it."""
import numpy as np

from blamm_gb300 import workloads


def random_case(d, seed: int) -> list[list[str]]:
    """A small case of fresh inputs: two species groups, N runs, lowercase stretches, ragged
    FASTA lines and blank lines, JASPAR or Cluster-Buster motifs, blocks of 20 kbp (the
    reference's default block height h = 1000 with w = 20: at h = 100 this OpenBLAS build
    rounds a few sgemm entries differently from motif-position order)."""
    rng = np.random.default_rng(seed)
    motifs = workloads.random_pfms(rng, 10, 4, 22)
    jaspar = seed % 2 == 0
    mfile = "motifs.jaspar" if jaspar else "motifs.cb"
    (workloads.write_jaspar if jaspar else workloads.write_cb)(str(d / mfile), motifs)
    workloads.write_settings(str(d / "settings.cnf"), w=20, h=1000)
    manifest = []
    for g, nfiles in (("groupA", 2), ("groupB", 1)):
        for f in range(nfiles):
            name = f"{g}_{f}.fa"
            with open(d / name, "wb") as out:
                for s in range(int(rng.integers(1, 4))):
                    seq = workloads.iid_bases(rng, int(rng.integers(2_000, 20_000)), [0.3, 0.2, 0.2, 0.3]).copy()
                    for _ in range(int(rng.integers(0, 4))):  # N runs
                        a = int(rng.integers(0, len(seq)))
                        seq[a:a + int(rng.integers(1, 300))] = ord("N")
                    for _ in range(int(rng.integers(0, 4))):  # lowercase (soft-masked) stretches
                        a = int(rng.integers(0, len(seq)))
                        seq[a:a + int(rng.integers(1, 500))] |= 0x20
                    out.write(f">{g}_seq{f}_{s} description\n".encode())
                    i = 0
                    while i < len(seq):
                        w = int(rng.integers(20, 100))
                        out.write(seq[i:i + w].tobytes() + b"\n")
                        if rng.random() < 0.02:
                            out.write(b"\n")
                        i += w
            manifest.append(f"{g}\t{name}\n")
    (d / "sequences.mf").write_text("".join(manifest))
    return [["dict", "sequences.mf"],
            ["hist", "-b", "120", mfile, "sequences.mf"],
            ["scan", "-rc", "-pt", "0.001", "-o", "occ_pt.txt", mfile, "sequences.mf"],
            ["scan", "-s", "-rt", "0.85", "-o", "occ_s.txt", mfile, "sequences.mf"],
            ["scan", "-rc", "-at", "5", "-o", "occ_at.txt", mfile, "sequences.mf"]]


def edge_case(d, crlf: bool) -> list[list[str]]:
    """FASTA edge cases: a header without bases, a sequence shorter than every motif, IUPAC
    codes and lowercase n inside a sequence, a soft-masked stretch, no newline at the end of
    the file; LF or CRLF line ends."""
    rng = np.random.default_rng(99)
    workloads.write_jaspar(str(d / "m.jaspar"), workloads.random_pfms(rng, 8, 4, 16))
    workloads.write_settings(str(d / "settings.cnf"), w=20, h=1000)
    eol = b"\r\n" if crlf else b"\n"
    seq = workloads.iid_bases(rng, 30_000, [0.3, 0.2, 0.2, 0.3]).copy()
    iupac = np.frombuffer(b"RYKMSWBDHVNn", np.uint8)
    for _ in range(40):
        a = int(rng.integers(0, len(seq)))
        seq[a:a + int(rng.integers(1, 5))] = iupac[int(rng.integers(0, len(iupac)))]
    seq[1000:1500] |= 0x20
    with open(d / "a.fa", "wb") as f:
        f.write(b">empty" + eol + b">short" + eol + b"ACG" + eol + b">iupac x y" + eol)
        for i in range(0, len(seq), 61):
            f.write(seq[i:i + 61].tobytes() + eol)
        f.write(b">last" + eol + workloads.iid_bases(rng, 500, [0.25] * 4).tobytes())
    (d / "sequences.mf").write_text("g\ta.fa\n")
    return [["dict", "sequences.mf"], ["hist", "-b", "80", "m.jaspar", "sequences.mf"],
            ["scan", "-rc", "-pt", "0.01", "-o", "occ_pt.txt", "m.jaspar", "sequences.mf"],
            ["scan", "-s", "-rc", "-rt", "0.8", "-o", "occ_s.txt", "m.jaspar", "sequences.mf"]]
