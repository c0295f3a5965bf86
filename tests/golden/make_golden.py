"""Generates the golden fixtures in this folder from the reference's own code
(oracle/_ref/libbvhref.so, compiled by oracle/ref/build_ref.py from the
reference's sources; only possible where those sources are present).

Each fixture ``reference_<case>.npz`` holds, for one seeded scene:

* the world-space triangles (``tris``) and the tree the reference's SAH
  builder made from them (CompactNodeManager<CompactNodeV3> records in the
  ``Bvh.export_compact`` layout: ``lo3 hi3 child_begin child_count prim_begin
  prim_count order48 depth prim_ids``), with ``N`` and ``L``;
* ray batches (``<batch>_rays``, [n, 8] = origin, tMax, direction, unused) and
  what the reference's CompactNodeManager::intersectImmediately returned for
  them: ``<batch>_prim`` (input triangle id, -1: none), ``<batch>_t``
  (Ray::tMax), ``<batch>_pos`` (Ray::surfacePosition), ``<batch>_occluded``,
  ``<batch>_counters`` (node visits, leaf visits, box tests, box hits,
  triangle tests, triangle hits per ray), ``<batch>_depth_hist`` (node / leaf
  visits per depth) and ``<batch>_fullness`` (childFullness,
  primitiveFullness summed over the batch; 17 bins each);
* for the ``wide`` batch, intersectWideAlternative over 256-ray packets with
  its per-step workgroup data (``wide_steps``, ``wide_step_count``).

The secondary rays are made from the reference's own closest hits (its
surface positions), one shadow ray and a few AO rays per hit, with the scene
generators of bvhraytracer_gb300.scenes.

Run from the repository root: ``python tests/golden/make_golden.py``.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from bvhraytracer_gb300 import sah_factor  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402
from oracle.ref.reference import ReferenceBvh  # noqa: E402

TREE_KEYS = ("lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48",
             "depth", "prim_ids")


def _normal(tris, prim):
    t = tris[prim].reshape(-1, 3, 3).astype(np.float64)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    return (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)


def _secondary(tris, prim, pos, rays, light, ao, ao_len, seed):
    """Shadow ray and AO rays per closest hit (bvhraytracer_gb300.scenes:
    origin offset 1e-3 along the face normal turned toward the incoming ray).
    Misses get none: the reference's renderer makes secondary rays only for
    hits, and its per-ray traversal has no notion of an inactive ray."""
    hit = prim >= 0
    nrm = _normal(tris, prim[hit])
    flip = np.einsum("ij,ij->i", nrm, rays[hit, 4:7]) > 0
    nrm[flip] *= -1
    p = pos[hit].astype(np.float32)
    return S.shadow_rays(p, nrm, light), S.ao_rays(p, nrm, ao, ao_len, seed=seed)


def _trace(ref, rays, shadow, prefix, out, packet=0):
    r = ref.trace(rays, shadow, packet=packet, step_cap=512 if packet else 0)
    out[prefix + "_rays"] = rays
    out[prefix + "_occluded"] = r["occluded"]
    out[prefix + "_counters"] = r["counters"]
    out[prefix + "_depth_hist"] = r["depth_hist"]
    full = np.zeros((2, 17), np.uint64)
    full[0, :r["child_fullness"].shape[0]] = r["child_fullness"]
    full[1, :r["prim_fullness"].shape[0]] = r["prim_fullness"]
    out[prefix + "_fullness"] = full
    if not shadow:
        out[prefix + "_prim"] = r["prim"]
        out[prefix + "_t"] = r["t"]
        out[prefix + "_pos"] = r["pos"]
    if packet:
        out[prefix + "_steps"] = r["steps"]
        out[prefix + "_step_count"] = r["step_count"]
    return r


def make_case(name, tris, n, l, primary, light, ao, ao_len, seed):
    ref = ReferenceBvh(tris, n, l, sah_factor(n, l))
    tree = ref.export_compact()
    out = {"tris": tris, "N": np.int32(n), "L": np.int32(l)}
    out.update({k: tree[k] for k in TREE_KEYS})
    r = _trace(ref, primary, False, "primary", out)
    sh, aos = _secondary(tris, r["prim"], r["pos"], primary, light, ao, ao_len, seed)
    _trace(ref, sh, True, "shadow", out)
    _trace(ref, aos, True, "ao", out)
    _trace(ref, primary[:2048], False, "wide", out, packet=256)
    path = HERE / f"reference_{name}.npz"
    np.savez_compressed(path, **out)
    return path


def main():
    paths = []
    # Terrain (the small configuration's generator at 32 x 32 quads), N4L4,
    # 96 x 96 primary rays from the same camera, one shadow ray per hit.
    tris = S.terrain(32, seed=0)
    centre = np.array([0.5, 0.0, 0.5])
    cam = S.camera_rays(centre + np.array([0.0, 1.5, 1.5]), centre, 96, 96)
    light = np.array([2.0, 3.0, 2.0], np.float32)
    paths.append(make_case("terrain32_N4L4", tris, 4, 4, cam, light, 2, 0.05, 3))
    # Clutter (40 objects), N8L8, and odd widths N3L5: 96 x 64 primary rays,
    # one shadow ray and 2 AO rays per hit.
    tris = S.clutter(40, seed=2)
    cam, target, light = S.clutter_viewpoints(40, seed=2)
    prim = S.camera_rays(cam, target, 96, 64)
    ao_len = 0.1 * S.scene_diagonal(tris)
    paths.append(make_case("clutter40_N8L8", tris, 8, 8, prim, light, 2, ao_len, 5))
    paths.append(make_case("clutter40_N3L5", tris, 3, 5, prim, light, 2, ao_len, 6))
    for p in paths:
        print(p, p.stat().st_size)


if __name__ == "__main__":
    main()
