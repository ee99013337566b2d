"""The drop-in `blamm` command line on the GPU against the reference's golden files.

Every command of each golden case (dict, hist, hist -e, scan with -pt/-rt/-at/-s,
both strands) must reproduce the reference's .dict, hist_*.dat/.gnu (theoretical
and empirical), PWMthresholds.txt and occurrence set byte for byte (occurrences
compared as sorted line sets).
"""
import pytest

import golden_cases as gc
from blamm_gb300._native import CLI_PATH

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", gc.CASES)
def test_cli_matches_reference(tmp_path, case):
    spec = gc.load(case)
    d = gc.stage(case, str(tmp_path))
    gc.run(CLI_PATH, d, spec)
    gc.compare(d, case, spec)


@pytest.mark.parametrize("mode", ["bf16", "fp32"])
@pytest.mark.parametrize("chunk", ["2999", "100000"])
def test_cli_modes_and_chunking(tmp_path, mode, chunk):
    """Small stream chunks (many chunk boundaries, overlaps) and every arithmetic mode
    give the same files."""
    case = "mixed"
    spec = gc.load(case)
    d = gc.stage(case, str(tmp_path))
    gc.run(CLI_PATH, d, spec, env={"BLAMM_CHUNK_BASES": chunk}, extra_scan=("-m", mode))
    gc.compare(d, case, spec)


def test_cli_motifs_longer_than_the_tensor_core_limit(tmp_path):
    """A bank with a 300-position motif: the CLI falls back to the plain FP32 GPU scan and
    writes the same files as the oracle's CLI (the reference's algorithm, any length)."""
    import os
    import subprocess

    import numpy as np

    import oracle
    from blamm_gb300 import workloads
    rng = np.random.default_rng(91)
    motifs = workloads.random_pfms(rng, 6, 5, 30) + [("LONG300", workloads.random_pfms(rng, 1, 300, 300)[0][1])]
    seqs = [(f"s{i}", workloads.iid_bases(rng, 120_000, [0.3, 0.2, 0.2, 0.3])) for i in range(2)]
    outs = {}
    for name, binary in (("ours", CLI_PATH), ("oracle", oracle.CLI_PATH)):
        d = tmp_path / name
        workloads.write_case(str(d), {"g": [("s.fa", seqs)]}, motifs)
        workloads.write_settings(str(d / "settings.cnf"))
        for cmd in (["dict", "sequences.mf"], ["hist", "motifs.jaspar", "sequences.mf"],
                    ["scan", "-rc", "-rt", "0.63", "motifs.jaspar", "sequences.mf"]):
            r = subprocess.run([binary] + cmd, cwd=d, capture_output=True, text=True)
            assert r.returncode == 0, (name, cmd, r.stdout[-500:], r.stderr[-500:])
        outs[name] = sorted(open(d / "occurrences.txt").read().splitlines())
    assert len(outs["ours"]) > 0 and outs["ours"] == outs["oracle"]
    assert any("LONG300" in line for line in outs["ours"])


@pytest.mark.parametrize("kind,arg", [("edge", False), ("edge", True), ("random", 0), ("random", 1)])
@pytest.mark.parametrize("piece", ["1", "268435456"])
def test_gpu_and_host_fasta_readers_write_the_same_files(tmp_path, kind, arg, piece):
    """The default FASTA reader (the text parsed on the GPU in pieces cut at header lines,
    kept on the device and scanned there) and the host reader (FastaStream, which the CPU
    suite pins to the reference's `dict` output on these cases) write byte-identical .dict,
    hist (theoretical and `hist -e`), PWMthresholds.txt and occurrence files.  Pieces of 1
    byte put every sequence in a piece of its own; chunks of 5000 bases cut the pieces
    further."""
    import os
    import subprocess

    from fresh_cases import edge_case, random_case
    make = edge_case if kind == "edge" else random_case
    outs = {}
    for name, env in (("host", {"BLAMM_FASTA_READER": "host"}),
                      ("gpu", {"BLAMM_INGEST_PIECE_BYTES": piece, "BLAMM_CHUNK_BASES": "5000"})):
        d = tmp_path / name
        d.mkdir()
        (d / "emp").mkdir()
        cmds = make(d, arg)
        mfile = next(c for c in cmds if c[0] == "hist")[-2]
        # empirical histograms of the first 9,000 bases: the limit falls inside a piece
        cmds.append(["hist", "-e", "-l", "9000", "-H", "emp", mfile, "sequences.mf"])
        for cmd in cmds:
            r = subprocess.run([CLI_PATH] + cmd, cwd=d, capture_output=True, text=True,
                               env=dict(os.environ, **env))
            assert r.returncode == 0, (name, cmd, r.stderr[-800:])
        outs[name] = d
    files = sorted(p.name for p in outs["host"].iterdir() if p.is_file())
    files += sorted("emp/" + p.name for p in (outs["host"] / "emp").iterdir())
    assert "sequences.mf.dict" in files and any(f.startswith("occ_") for f in files)
    assert any(f.startswith("emp/hist_") for f in files)
    for f in files:
        assert (outs["host"] / f).read_bytes() == (outs["gpu"] / f).read_bytes(), f


def test_gpu_reader_rejects_sequence_data_before_a_header(tmp_path):
    """The GPU reader stops like the reference's dict module (FastaBatch::getNextLine throws,
    blstools.cpp:93-101 exits 1)."""
    import subprocess
    (tmp_path / "bad.fa").write_text("ACGT\n>s1\nACGTACGT\n")
    (tmp_path / "bad.mf").write_text("sp\tbad.fa\n")
    r = subprocess.run([CLI_PATH, "dict", "bad.mf"], cwd=tmp_path, capture_output=True)
    assert r.returncode == 1
    assert b"Input file does not appear to be in fasta format" in r.stderr + r.stdout
