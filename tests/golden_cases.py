"""Running a golden case (tests/golden/<case>) with some `blamm`-compatible binary."""
from __future__ import annotations

import gzip
import json
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = sorted(d for d in os.listdir(GOLDEN) if os.path.isfile(os.path.join(GOLDEN, d, "case.json")))


def load(case: str) -> dict:
    with open(os.path.join(GOLDEN, case, "case.json")) as f:
        return json.load(f)


def stage(case: str, tmp: str) -> str:
    """Copy the case inputs (not the expected outputs) into a fresh directory."""
    src = os.path.join(GOLDEN, case)
    dst = os.path.join(tmp, case)
    shutil.copytree(src, dst, ignore=shutil.ignore_patterns("expected", "case.json"))
    for root, _, files in os.walk(dst):  # inputs stored gzip-compressed are inflated
        for f in files:
            if f.endswith(".gz"):
                p = os.path.join(root, f)
                with gzip.open(p, "rb") as fi, open(p[:-3], "wb") as fo:
                    shutil.copyfileobj(fi, fo)
                os.remove(p)
    os.makedirs(os.path.join(dst, "emp"), exist_ok=True)
    return dst


def run(binary: str, d: str, spec: dict, skip=(), env=None, extra_scan=()) -> None:
    for cmd in spec["commands"]:
        if any(s(cmd) for s in skip):
            continue
        args = [binary] + cmd
        if cmd[0] == "scan" and extra_scan:
            args = [binary, "scan", *extra_scan] + cmd[1:]
        res = subprocess.run(args, cwd=d, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                             env=dict(os.environ, **(env or {})))
        assert res.returncode == 0, f"{args} failed:\n{res.stderr.decode()[-2000:]}"


def sorted_lines(path: str) -> list[bytes]:
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rb") as f:
        return sorted(f.read().splitlines(keepends=True))


def compare(d: str, case: str, spec: dict, what=("dict", "hist", "thresholds", "occ", "emp")) -> None:
    exp = os.path.join(GOLDEN, case, "expected")
    for f in sorted(os.listdir(exp)):
        e = os.path.join(exp, f)
        if f.endswith(".gz"):  # a compressed expected file: compared with the uncompressed output
            f = f[:-3]
        g = os.path.join(d, f)
        if f == "emp":
            if "emp" in what:
                for h in sorted(os.listdir(e)):
                    assert _same_bytes(os.path.join(e, h), os.path.join(d, "emp", h)), f"emp/{h} differs"
            continue
        if f.endswith(".dict"):
            if "dict" in what:
                assert _same_bytes(e, g), f"{f} differs"
        elif f.startswith("hist_"):
            if "hist" in what:
                assert _same_bytes(e, g), f"{f} differs"
        elif f == "PWMthresholds.txt":
            if "thresholds" in what:
                assert sorted_lines(e) == sorted_lines(g), "PWMthresholds.txt differs"
        elif f in spec["outputs"]:
            if "occ" in what:
                a, b = sorted_lines(e), sorted_lines(g)
                if a != b:
                    sa, sb = set(a), set(b)
                    raise AssertionError(f"{f}: {len(a)} vs {len(b)} lines; missing {sorted(sa - sb)[:3]} "
                                         f"extra {sorted(sb - sa)[:3]}")


def _same_bytes(a: str, b: str) -> bool:
    if not os.path.exists(b):
        return False
    with open(a, "rb") as fa, open(b, "rb") as fb:
        return fa.read() == fb.read()
