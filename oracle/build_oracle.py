"""Builds the CPU oracle (test infrastructure) from oracle/bvh_oracle.c and
oracle/sah_builder.c:

* oracle/_build/liboracle.so — the scalar restatement (the oracle proper): gcc -O2
  with -ffp-contract=off (no FMA contraction, so float results match the
  reference's scalar code on x86-64 and aarch64 alike) and OpenMP;
* oracle/_build/libcpubaseline.so — the timed CPU baseline: the same source
  with -DORACLE_SIMD at -O3, where the ISPC kernels' gang lanes run as 4-wide
  GCC vectors (SSE on x86-64, NEON on aarch64). No -march / -mcpu flag: the
  library must compile and give the same results on x86 and Arm; the
  4-wide vectors are in both base instruction sets. Its results equal the
  scalar build's bit for bit (tests/test_cpu_baseline.py).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRCS = [HERE / "bvh_oracle.c", HERE / "sah_builder.c"]
OUT = HERE / "_build" / "liboracle.so"
OUT_SIMD = HERE / "_build" / "libcpubaseline.so"


def _compile(out: Path, flags: list[str]) -> Path:
    out.parent.mkdir(parents=True, exist_ok=True)
    if out.exists() and all(out.stat().st_mtime > s.stat().st_mtime for s in SRCS):
        return out
    cc = os.environ.get("CC", "gcc")
    tmp = out.with_suffix(".so.tmp")
    cmd = [cc] + flags + ["-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
                          "-fno-fast-math", "-fopenmp"] + [str(s) for s in SRCS] + [
                              "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    os.replace(tmp, out)
    return out


def build() -> Path:
    """Both libraries; returns the scalar oracle's path."""
    _compile(OUT_SIMD, ["-O3", "-DORACLE_SIMD"])
    return _compile(OUT, ["-O2"])


def build_baseline() -> Path:
    return _compile(OUT_SIMD, ["-O3", "-DORACLE_SIMD"])


if __name__ == "__main__":
    print(build(), build_baseline())
