"""The oracle is pinned to the reference: same files on the golden cases (CPU only).

The golden outputs were written by the compiled reference (tests/golden/make_golden.py);
where the reference's sources are mounted, the reference's own example data is
run through both programs as well.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_cases as gc
import oracle
from bankutil import make_bank, make_stream, same_hits
from fresh_cases import edge_case, random_case


@pytest.mark.parametrize("case", gc.CASES)
def test_oracle_cli_matches_reference_fixtures(tmp_path, case):
    spec = gc.load(case)
    d = gc.stage(case, str(tmp_path))
    # the oracle restates the theoretical histogram only; empirical ones are checked on the GPU
    gc.run(oracle.CLI_PATH, d, spec, skip=[lambda c: c[0] == "hist" and "-e" in c])
    gc.compare(d, case, spec, what=("dict", "hist", "thresholds", "occ"))


import oracle_build  # oracle/oracle_build.py

EXAMPLE = os.path.join(oracle_build.reference_dir(), "example")


@pytest.mark.skipif(not (os.path.isdir(EXAMPLE) and os.path.exists(oracle.REF_CLI_PATH)),
                    reason="reference example / binary only in the development container")
def test_oracle_matches_reference_on_its_example(tmp_path):
    outs = {}
    for name, binary in (("ref", oracle.REF_CLI_PATH), ("orc", oracle.CLI_PATH)):
        d = tmp_path / name
        shutil.copytree(EXAMPLE, d)
        for p in d.rglob("*"):
            p.chmod(0o755 if p.is_dir() else 0o644)
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
        for cmd in (["dict", "sequences.mf"], ["hist", "motifs.jaspar", "sequences.mf"],
                    ["scan", "-rc", "-pt", "0.0001", "motifs.jaspar", "sequences.mf"]):
            subprocess.run([binary] + cmd, cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
        outs[name] = d
    for f in ["sequences.mf.dict"] + sorted(p.name for p in outs["ref"].glob("hist_*")):
        assert (outs["ref"] / f).read_bytes() == (outs["orc"] / f).read_bytes(), f
    for f in ("occurrences.txt", "PWMthresholds.txt"):
        a = sorted((outs["ref"] / f).read_bytes().splitlines())
        b = sorted((outs["orc"] / f).read_bytes().splitlines())
        assert a == b, f
    assert len(a) > 0


def _differential(tmp_path, make) -> None:
    """Run the compiled reference and the oracle on the same fresh case; they must write the
    same dictionary, histograms, thresholds and occurrences."""
    outs = {}
    for name, binary in (("ref", oracle.REF_CLI_PATH), ("orc", oracle.CLI_PATH)):
        d = tmp_path / name
        d.mkdir()
        cmds = make(d)
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
        for cmd in cmds:
            subprocess.run([binary] + cmd, cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
        outs[name] = d
    ref, orc = outs["ref"], outs["orc"]
    hists = sorted(p.name for p in ref.glob("hist_*"))
    assert len(hists) > 0
    for f in ["sequences.mf.dict"] + hists:
        assert (ref / f).read_bytes() == (orc / f).read_bytes(), f
    occ = sorted(p.name for p in ref.glob("occ_*.txt"))
    assert len(occ) == sum(c[0] == "scan" for c in cmds)
    for f in ["PWMthresholds.txt"] + occ:
        a = sorted((ref / f).read_bytes().splitlines())
        b = sorted((orc / f).read_bytes().splitlines())
        assert a == b, f"{f}: {len(a)} vs {len(b)} lines"
        assert len(a) > 0, f


NEEDS_REF = pytest.mark.skipif(not os.path.exists(oracle.REF_CLI_PATH),
                               reason="reference binary only in the development container")


@NEEDS_REF
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_matches_reference_on_random_cases(tmp_path, seed):
    _differential(tmp_path, lambda d: random_case(d, seed))


@NEEDS_REF
@pytest.mark.parametrize("crlf", [False, True])
def test_oracle_matches_reference_on_fasta_edge_cases(tmp_path, crlf):
    _differential(tmp_path, lambda d: edge_case(d, crlf))


def test_blas_port_equals_sequential_scan():
    """OpenBLAS sums the one-hot products in motif-position order: the reference's
    BLAS loop and the sequential FP32 scorer agree bit for bit."""
    P, lens, thr = make_bank(21, 48, 5, 30, rel=0.85)
    bases, runs = make_stream(22, 600_000, nruns=30, lower_frac=0.03)
    tiles = oracle.matrix_tiles(lens, 4096)
    ok, msg = same_hits(oracle.scan_blas(bases, runs, P, lens, thr, tiles, 1000, 250, 8),
                        oracle.scan(bases, runs, P, lens, thr))
    assert ok, msg


def test_planted_mistake_is_caught():
    """A one-ulp change in one P entry must change the hit set the checker sees."""
    P, lens, thr = make_bank(23, 16, 8, 14, rel=0.85)
    bases, runs = make_stream(24, 200_000)
    good = oracle.scan(bases, runs, P, lens, thr)
    hit = good[len(good) // 2]
    thr2 = thr.copy()
    thr2[hit["col"]] = np.nextafter(hit["score"], np.float32(np.inf))  # just above one score
    bad = oracle.scan(bases, runs, P, lens, thr2)
    ok, _ = same_hits(good, bad)
    assert not ok
