"""Cached scenes, BVHs and oracle views shared by the tests."""
from __future__ import annotations

import functools

import numpy as np

import bvhraytracer_gb300 as pkg
from bvhraytracer_gb300 import scenes as S
from oracle import oracle as O


@functools.lru_cache(maxsize=None)
def terrain_case():
    tris, rays, light = S.terrain_workload()
    return tris, rays, light


@functools.lru_cache(maxsize=None)
def clutter_tris(n_objects: int = 120, seed: int = 3):
    return S.clutter(n_objects, seed)


@functools.lru_cache(maxsize=None)
def bvh(kind: str, n: int, l: int, **kw):
    if kind == "terrain":
        tris = terrain_case()[0]
    elif kind.startswith("clutter"):
        tris = clutter_tris(int(kind[7:] or 120))
    else:
        raise KeyError(kind)
    b = pkg.Bvh(tris, n, l, **kw)
    return tris, b, O.CompactView(b.export_compact())


def clutter_rays(tris: np.ndarray, n_objects: int = 120, res=(96, 64)):
    return S.clutter_camera(n_objects, *res, seed=3)


def secondary(tris, rays, prims, light, ao_samples=2, length=None, seed=7):
    m, p, nrm = S.surface(tris, rays, prims)
    sh = S.shadow_rays(p, nrm, light)
    ln = length if length is not None else 0.1 * S.scene_diagonal(tris)
    ao = S.ao_rays(p, nrm, ao_samples, ln, seed=seed)
    return sh, ao
