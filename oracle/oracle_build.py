"""Builds the test infrastructure: the CPU oracle (liboracle.so, the oracle CLI) and, where the
reference's sources are found, the unmodified reference binary (oracle/_ref/blamm) that pins
the oracle.  Not part of the product build: the tests, __graft_entry__ and bench.py's CPU legs
call it.

The reference's location: $BLAMM_REFERENCE_DIR, else the default the build recipe
(oracle/build_ref.sh) declares.
"""
from __future__ import annotations

import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_dir() -> str:
    """Root of the reference's source tree (it may not exist on this machine)."""
    env = os.environ.get("BLAMM_REFERENCE_DIR")
    if env:
        return env
    with open(os.path.join(HERE, "build_ref.sh")) as f:
        m = re.search(r"^DEFAULT_REF=(\S+)$", f.read(), flags=re.M)
    return m.group(1) if m else ""


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed: " + " ".join(cmd) + "\n" + res.stdout)


def build(force: bool = False, with_reference: bool = True) -> None:
    import platform
    out = os.path.join(HERE, "_build")
    os.makedirs(out, exist_ok=True)
    stamp = os.path.join(out, ".arch")  # objects built on another architecture are rebuilt
    if not os.path.exists(stamp) or open(stamp).read().strip() != platform.machine():
        force = True
    if force:
        _run(["make", "-s", "-C", HERE, "clean"])
    _run(["make", "-s", "-C", HERE])
    with open(stamp, "w") as f:
        f.write(platform.machine() + "\n")
    ref = reference_dir()
    ref_bin = os.path.join(HERE, "_ref", "blamm")
    if with_reference and ref and os.path.isdir(os.path.join(ref, "src")) and (force or not os.path.exists(ref_bin)):
        _run(["bash", os.path.join(HERE, "build_ref.sh"), ref])


if __name__ == "__main__":
    import sys
    build(force="--force" in sys.argv)
