"""Compiles the reference's own instrumented renderer code into
oracle/_ref/libbvhref.so — TEST INFRASTRUCTURE (the recipe behind
oracle/ref/reference.py; only tests/ and tests/golden/make_golden.py use it).

The sources are the reference's, read from /root/reference/src:

    src/ray.cpp                              Ray (counters, normalised direction)
    src/primitives/triangle.cpp              Triangle::intersect (watertight)
    src/accelerationStructure/aabb.cpp       Aabb::recursiveBvh (SAH builder)
    src/accelerationStructure/node.cpp       Node, traverse orders
    src/accelerationStructure/bvh.cpp        Bvh, bvhAnalysis (NodeAnalysis tree)
    src/accelerationStructure/compactNode.cpp  CompactNodeManager traversals
    src/lodepng/lodepng.cpp                  (linked by bvh.cpp's image writer)

plus oracle/ref/ref_driver.cpp (this repository's C entry points around
them). The reference is written for MSVC with GLM; it is compiled here with
g++ 13 and a GLM stand-in (oracle/ref_shim/glm, written for this repository),
after four textual fixes that g++ needs, applied to a temporary copy of the
sources (nothing is written under /root/reference, and no reference source
enters this repository):

1. aabb.h:205-238 defines Aabb's overrides as ``inline void
   Node::sweepRight() override`` inside class Aabb, a qualified name MSVC
   accepts and g++ rejects: the ``Node::`` qualifier is dropped (same
   meaning: Aabb's override of Node::sweepRight and friends).
2. bvh.cpp:26 includes ``"..\\timing.h"``: the backslash becomes a slash.
3. util.h:13 selects the MSVC definition of MachineEpsilon (a double
   expression, so pbrt's gamma(n) is evaluated in double as the reference's
   MSVC build does) with ``#ifdef _MSC_VER``: that branch is taken here too.
4. MSVC's standard headers make <memory>'s shared_ptr and the C library's
   global ``isnan`` visible through <iostream> / <cmath>; libstdc++'s do not,
   so every file is compiled with ``-include memory -include math.h``.

``std::sort(std::execution::par_unseq, ...)`` (aabb.h:63-66) runs through
libstdc++'s serial PSTL back end (no TBB here): an introsort, so the order of
triangles with equal centres can differ from this repository's stable sort.
Trees are therefore compared on scenes whose triangle centres are distinct
per axis; traversal results are compared on the reference's own tree.

Run ``python -m oracle.ref.build_ref`` (or call ``build()``); it returns the
library path, or raises if the reference sources are not present.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF_SRC = Path(os.environ.get("BVHREF_SOURCES", "/root/reference/src"))
SHIM = HERE.parent / "ref_shim"
DRIVER = HERE / "ref_driver.cpp"
OUT = HERE.parent / "_ref" / "libbvhref.so"

UNITS = ["ray.cpp", "primitives/triangle.cpp", "accelerationStructure/aabb.cpp",
         "accelerationStructure/node.cpp", "accelerationStructure/bvh.cpp",
         "accelerationStructure/compactNode.cpp", "lodepng/lodepng.cpp"]
CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w",
            "-include", "memory", "-include", "math.h"]


def available() -> bool:
    return (REF_SRC / "accelerationStructure" / "compactNode.cpp").exists()


def _fixes(tree: Path) -> None:
    """The four g++ fixes listed in the module docstring."""
    aabb = tree / "accelerationStructure" / "aabb.h"
    text = aabb.read_text()
    n = text.count("inline void Node::sweep")
    if n != 4:
        raise RuntimeError(f"aabb.h: expected 4 qualified sweep overrides, found {n}")
    aabb.write_text(text.replace("inline void Node::sweep", "inline void sweep"))
    bvh = tree / "accelerationStructure" / "bvh.cpp"
    text = bvh.read_text()
    if '#include "..\\timing.h"' not in text:
        raise RuntimeError("bvh.cpp: backslash include not found")
    bvh.write_text(text.replace('#include "..\\timing.h"', '#include "../timing.h"'))
    util = tree / "util.h"
    text = util.read_text()
    if "#ifdef _MSC_VER\n#define MachineEpsilon" not in text.replace("\r\n", "\n"):
        raise RuntimeError("util.h: MSVC MachineEpsilon branch not found")
    util.write_text(text.replace("#ifdef _MSC_VER", "#if 1 /* the MSVC branch */", 1))


def _stale() -> bool:
    if not OUT.exists():
        return True
    t = OUT.stat().st_mtime
    deps = [DRIVER, Path(__file__)] + list(SHIM.rglob("*.hpp"))
    deps += [REF_SRC / u for u in UNITS]
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def build(force: bool = False) -> Path:
    if not available():
        raise FileNotFoundError(f"reference sources not found at {REF_SRC}")
    if not force and not _stale():
        return OUT
    cxx = os.environ.get("CXX", "g++")
    OUT.parent.mkdir(parents=True, exist_ok=True)
    with tempfile.TemporaryDirectory(prefix="bvhref_") as tmp:
        tree = Path(tmp) / "src"
        shutil.copytree(REF_SRC, tree, ignore=shutil.ignore_patterns(
            "tinyGltf", "catch2", "Catch2Testing", "ISPC", "*.vcxproj*"))
        _fixes(tree)
        inc = ["-I", str(SHIM), "-I", str(tree)]
        jobs = [(tree / u, Path(tmp) / (u.replace("/", "_") + ".o")) for u in UNITS]
        jobs.append((DRIVER, Path(tmp) / "ref_driver.o"))

        def compile_one(job):
            src, obj = job
            cmd = [cxx] + CXXFLAGS + inc + ["-c", str(src), "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
            return obj

        with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
            objs = list(ex.map(compile_one, jobs))
        tmp_out = OUT.with_suffix(".so.tmp")
        cmd = [cxx, "-shared", "-Wl,--no-undefined", "-o", str(tmp_out)] + [str(o) for o in objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference link failed:\n" + r.stderr)
        os.replace(tmp_out, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
