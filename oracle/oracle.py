"""ctypes wrapper of the CPU oracle (oracle/bvh_oracle.c) — TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module. Parity status: the instrumented profile is pinned
against the reference's own code compiled here (oracle/ref/) and the fixtures
it generated (tests/golden/); the fast (ISPC) profile is not, see the header
of bvh_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from .build_oracle import build

_P = C.c_void_p


class _Compact(C.Structure):
    _fields_ = [("n_nodes", C.c_uint64)] + [(k, _P) for k in (
        "lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48",
        "depth", "prim_ids", "prim_tri9")]


class _Fast(C.Structure):
    _fields_ = [("n_nodes", C.c_uint64), ("gang", C.c_int32), ("node_memory", C.c_int32),
                ("leaf_memory", C.c_int32)] + [(k, _P) for k in (
                    "bounds", "begin", "order", "child_type", "tri_points")]


_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(str(build()))
            L.oracle_trace_instrumented.restype = C.c_int
            L.oracle_trace_instrumented.argtypes = [C.POINTER(_Compact), _P, C.c_uint64, C.c_int,
                                                    _P, _P, _P, _P, C.c_int, _P]
            L.oracle_trace_instrumented_stream.restype = C.c_int
            L.oracle_trace_instrumented_stream.argtypes = [C.POINTER(_Compact), _P, C.c_uint64,
                                                           C.c_int, C.c_int, _P, _P, _P, _P, _P]
            L.oracle_trace_instrumented_stream_steps.restype = C.c_int
            L.oracle_trace_instrumented_stream_steps.argtypes = [
                C.POINTER(_Compact), _P, C.c_uint64, C.c_int, C.c_int, _P, _P, _P, _P, C.c_int,
                _P, _P, C.c_int, _P]
            L.oracle_trace_fast.restype = C.c_int
            L.oracle_trace_fast.argtypes = [C.POINTER(_Fast), C.POINTER(_Compact), _P, C.c_uint64,
                                            C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P,
                                            C.c_int]
            L.oracle_hit_points.restype = None
            L.oracle_hit_points.argtypes = [_P, _P, C.c_uint64, _P]
            L.oracle_fp64_pairs.restype = None
            L.oracle_fp64_pairs.argtypes = [_P, _P, C.c_uint64, C.c_int, _P]
            L.oracle_aabb_intersect_calls.restype = None
            L.oracle_aabb_intersect_calls.argtypes = [C.c_int32, _P, _P, _P, _P, _P, C.c_uint64]
            L.oracle_tri_intersect_calls.restype = None
            L.oracle_tri_intersect_calls.argtypes = [C.c_int32, C.c_int32, _P, _P, _P, _P,
                                                     C.c_uint64]
            L.oracle_tri_any_hit_calls.restype = None
            L.oracle_tri_any_hit_calls.argtypes = [C.c_int32, _P, _P, _P, _P, C.c_uint64]
            _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class CompactView:
    """Keeps the exported CompactNodeV3 arrays alive next to the C view."""

    def __init__(self, arrays: dict):
        self.a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        self.c = _Compact(self.a["child_count"].shape[0], *[_p(self.a[k]) for k in (
            "lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48",
            "depth", "prim_ids", "prim_tri9")])


class FastView:
    def __init__(self, arrays: dict):
        self.a = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v)
                  for k, v in arrays.items()}
        self.c = _Fast(self.a["begin"].shape[0], self.a["gang"], self.a["node_memory"],
                       self.a["leaf_memory"], *[_p(self.a[k]) for k in (
                           "bounds", "begin", "order", "child_type", "tri_points")])


def trace_instrumented(view: CompactView, rays: np.ndarray, shadow: bool, packet: int = 0,
                       counters: bool = True, use_distance: bool = False) -> dict:
    """CompactNodeManager::intersectImmediately(ray, use_distance) (packet ==
    0) or intersectWideAlternative over packets of ``packet`` rays. With
    ``counters``: per-ray counters, per-depth node / leaf visits
    (``depth_hist``) and Ray::childFullness / primitiveFullness summed over
    the rays (``fullness`` [2, 17]: visits of nodes with c children, of leaves
    with c triangles)."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    hits = None if shadow else np.zeros((n, 4), np.float32)
    occ = np.zeros(n, np.uint8) if shadow else None
    ctr = np.zeros((n, 8), np.uint32) if counters else None
    hist = np.zeros((2, 64), np.uint64) if counters else None
    full = np.zeros((2, 17), np.uint64) if counters else None
    if packet and use_distance:
        raise ValueError("use_distance is a per-ray traversal")
    if packet:
        rc = lib().oracle_trace_instrumented_stream(C.byref(view.c), _p(rays), n, int(shadow),
                                                     packet, _p(hits), _p(occ), _p(ctr), _p(hist),
                                                     _p(full))
    else:
        rc = lib().oracle_trace_instrumented(C.byref(view.c), _p(rays), n, int(shadow), _p(hits),
                                             _p(occ), _p(ctr), _p(hist), int(use_distance),
                                             _p(full))
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return {"hits": hits, "occluded": occ, "counters": ctr, "depth_hist": hist, "fullness": full}


def trace_fast(fview: FastView, cview: CompactView, rays: np.ndarray, any_hit: bool,
               packet: int = 0, threads: int = 0, counters: bool = True,
               outputs: bool = True, use_distance: bool = False) -> dict:
    """FastNodeManager::intersect / intersectSecondary (packet == 0) or the
    WideAlternative stream versions, with ISPC gang-lane semantics;
    ``use_distance``: intersectSaveDistance (per ray)."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    hits = np.zeros((n, 4), np.float32) if (outputs and not any_hit) else None
    occ = np.zeros(n, np.uint8) if (outputs and any_hit) else None
    li = np.zeros(n, np.int32) if (outputs and not any_hit) else None
    ti = np.zeros(n, np.int8) if (outputs and not any_hit) else None
    ctr = np.zeros((n, 8), np.uint32) if counters else None
    hist = np.zeros((2, 64), np.uint64) if counters else None
    rc = lib().oracle_trace_fast(C.byref(fview.c), C.byref(cview.c), _p(rays), n, int(any_hit),
                                 packet, threads, _p(hits), _p(occ), _p(li), _p(ti), _p(ctr),
                                 _p(hist), int(use_distance))
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return {"hits": hits, "occluded": occ, "leaf_index": li, "tri_index": ti, "counters": ctr,
            "depth_hist": hist}


def trace_instrumented_steps(view: CompactView, rays: np.ndarray, shadow: bool, packet: int,
                             step_cap: int, wide_alternative: bool = True) -> dict:
    """intersectWideAlternative over packets of ``packet`` rays with the
    per-step workgroup data (bvh_oracle.c: stream_impl): ``steps`` [packets,
    step_cap, 5] (node work, unique nodes, leaf work, unique leaves,
    terminations) and ``step_count`` [packets], plus hits / occlusion and
    counters."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = rays.shape[0]
    npk = -(-n // packet)
    hits = None if shadow else np.zeros((n, 4), np.float32)
    occ = np.zeros(n, np.uint8) if shadow else None
    ctr = np.zeros((n, 8), np.uint32)
    hist = np.zeros((2, 64), np.uint64)
    steps = np.zeros((npk, step_cap, 5), np.uint32)
    count = np.zeros(npk, np.uint32)
    full = np.zeros((2, 17), np.uint64)
    rc = lib().oracle_trace_instrumented_stream_steps(
        C.byref(view.c), _p(rays), n, int(shadow), packet, _p(hits), _p(occ), _p(ctr), _p(hist),
        step_cap, _p(steps), _p(count), int(wide_alternative), _p(full))
    if rc:
        raise RuntimeError(f"oracle error {rc}")
    return {"hits": hits, "occluded": occ, "counters": ctr, "depth_hist": hist, "steps": steps,
            "step_count": count, "fullness": full}


def hit_points(rays: np.ndarray, tri9: np.ndarray) -> np.ndarray:
    """Triangle::intersect's hit point b0 p0 + b1 p1 + b2 p2 of each (ray,
    triangle) pair, instrumented profile (NaN where the pair does not hit)."""
    rays = np.ascontiguousarray(rays, np.float32)
    tri9 = np.ascontiguousarray(tri9, np.float32)
    out = np.zeros((rays.shape[0], 3), np.float32)
    lib().oracle_hit_points(_p(rays), _p(tri9), rays.shape[0], _p(out))
    return out


def fp64_pairs(rays: np.ndarray, tri9: np.ndarray, normalise: bool) -> np.ndarray:
    """Double-precision (t, b1, b2) of each (ray, triangle) pair."""
    rays = np.ascontiguousarray(rays, np.float32)
    tri9 = np.ascontiguousarray(tri9, np.float32)
    out = np.zeros((rays.shape[0], 3), np.float64)
    lib().oracle_fp64_pairs(_p(rays), _p(tri9), rays.shape[0], int(normalise), _p(out))
    return out


def aabb_intersect_calls(n: int, bounds: np.ndarray, offsets: np.ndarray, fastrays: np.ndarray,
                         distances: np.ndarray):
    """aabbIntersect{n} per call (bvh_oracle.c: oracle_aabb_intersect_calls):
    returns (result [count] u8, distances [count, n] with t0 written at hit
    lanes of the given array)."""
    bounds = np.ascontiguousarray(bounds, np.float32)
    offsets = np.ascontiguousarray(offsets, np.uint32)
    fastrays = np.ascontiguousarray(fastrays, np.float32)
    dist = np.array(distances, np.float32, copy=True, order="C")
    res = np.zeros(offsets.shape[0], np.uint8)
    lib().oracle_aabb_intersect_calls(n, _p(bounds), _p(offsets), _p(fastrays), _p(dist),
                                      _p(res), offsets.shape[0])
    return res, dist


def tri_intersect_calls(l: int, gang: int, tri: np.ndarray, ids: np.ndarray,
                        fastrays: np.ndarray):
    """triIntersect{l} per call: returns (in-leaf index or -1, the FastRay
    records with tMax lowered on hits)."""
    tri = np.ascontiguousarray(tri, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    fr = np.array(fastrays, np.float32, copy=True, order="C")
    res = np.zeros(ids.shape[0], np.int32)
    lib().oracle_tri_intersect_calls(l, gang, _p(tri), _p(ids), _p(fr), _p(res), ids.shape[0])
    return res, fr


def tri_any_hit_calls(l: int, tri: np.ndarray, ids: np.ndarray, fastrays: np.ndarray):
    """triAnyHit{l} per call: returns [count] u8."""
    tri = np.ascontiguousarray(tri, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    fr = np.ascontiguousarray(fastrays, np.float32)
    res = np.zeros(ids.shape[0], np.uint8)
    lib().oracle_tri_any_hit_calls(l, _p(tri), _p(ids), _p(fr), _p(res), ids.shape[0])
    return res
