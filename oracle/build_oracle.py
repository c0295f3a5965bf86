"""Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

gcc with -ffp-contract=off (no FMA contraction, so float results match the
reference's scalar code on x86-64 and aarch64 alike) and OpenMP.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "bvh_oracle.c"
OUT = HERE / "_build" / "liboracle.so"


def build() -> Path:
    OUT.parent.mkdir(parents=True, exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime > SRC.stat().st_mtime:
        return OUT
    cc = os.environ.get("CC", "gcc")
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build())
