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
