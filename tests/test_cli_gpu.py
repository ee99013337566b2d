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
