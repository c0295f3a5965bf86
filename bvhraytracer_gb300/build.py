"""In-tree build of libbvhgpu.so (host C++ + sm_103a CUDA) with nvcc and g++.

Translation units compile in parallel; objects are reused when their source
and the headers are older than the object. Output: ``bvhraytracer_gb300/_build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libbvhgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Bit-exact float semantics: no FMA contraction, IEEE division / square root,
# denormals kept.
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    f"-I{INCLUDE}", f"-I{CSRC}",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
             f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build bvhgpu")
    return cand


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, defines: tuple = (), out_dir: Path | None = None) -> Path:
    """Compiles every translation unit and links libbvhgpu.so; returns its path.

    ``defines`` (e.g. ``("BVHGPU_PERSIST_MIN_BLOCKS=6",)``) and ``out_dir``
    build a variant of the library elsewhere, for tuning experiments.
    """
    build_dir = Path(out_dir) if out_dir else BUILD
    lib_path = build_dir / "libbvhgpu.so"
    build_dir.mkdir(parents=True, exist_ok=True)
    extra = [f"-D{d}" for d in defines]
    headers = list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "bvhgpu.h"]
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = build_dir / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + extra + ["-c", str(src), "-o", str(obj)])
    cxx = os.environ.get("CXX", "g++")
    for src in sorted(CSRC.glob("*.cpp")):
        obj = build_dir / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([cxx] + CXX_FLAGS + [f"-I{_cuda_include()}", "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if jobs or _stale(lib_path, objs):
        tmp = build_dir / "libbvhgpu.so.tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] +
             ["-Xcompiler", "-pthread"])
        os.replace(tmp, lib_path)
    if verbose:
        print(f"built {lib_path}")
    return lib_path


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
