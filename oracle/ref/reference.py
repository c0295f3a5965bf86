"""ctypes binding of oracle/_ref/libbvhref.so — TEST INFRASTRUCTURE.

The library is the reference's own SAH builder and instrumented traversal
(CompactNodeManager<CompactNodeV3>, Triangle::intersect, Ray) compiled by
oracle/ref/build_ref.py from the reference's sources. It exists only where
those sources are present; it pins the oracle restatement (bvh_oracle.c) and,
through the committed fixtures of tests/golden/, the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_ref import available, build  # noqa: F401

_P = C.c_void_p
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        L.bvhref_build.restype = C.c_int
        L.bvhref_build.argtypes = [_P, C.c_uint64, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                   C.c_float, C.c_int32, C.POINTER(_P)]
        L.bvhref_free.restype = None
        L.bvhref_free.argtypes = [_P]
        L.bvhref_sizes.restype = None
        L.bvhref_sizes.argtypes = [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_int32)]
        L.bvhref_export.restype = None
        L.bvhref_export.argtypes = [_P] * 7 + [_P, C.c_int32, _P, _P]
        L.bvhref_trace.restype = C.c_int
        L.bvhref_trace.argtypes = [_P, _P, C.c_uint64, C.c_int32, C.c_int32, C.c_int32,
                                   _P, _P, _P, _P, _P, _P, _P, C.c_int32, _P, _P, _P, _P,
                                   C.c_int32]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class ReferenceBvh:
    """The reference's Bvh + CompactNodeManager<CompactNodeV3> over world-space
    triangles ``[T, 9]`` (input order = scene-loader order)."""

    def __init__(self, tris, branching: int, leaf_size: int, sah: float, *,
                 leaf_split_option: int = 1, sort_each_split: bool = True, node_order: int = 0):
        self.tris = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 9))
        self.branching, self.leaf_size = branching, leaf_size
        h = _P()
        rc = lib().bvhref_build(_p(self.tris), self.tris.shape[0], branching, leaf_size,
                                leaf_split_option, int(sort_each_split), sah, node_order,
                                C.byref(h))
        if rc:
            raise RuntimeError(f"reference build failed ({rc})")
        self._h = h
        n, t, d = C.c_uint64(), C.c_uint64(), C.c_int32()
        lib().bvhref_sizes(h, C.byref(n), C.byref(t), C.byref(d))
        self.n_nodes, self.n_prims, self.depth = n.value, t.value, d.value

    def __del__(self):
        if getattr(self, "_h", None):
            lib().bvhref_free(self._h)
            self._h = None

    def export_compact(self) -> dict:
        """The CompactNodeV3 records in the layout of
        ``bvhraytracer_gb300.Bvh.export_compact`` (order48: 3 axes x 16)."""
        n, t = self.n_nodes, self.n_prims
        out = {"lo3": np.zeros((n, 3), np.float32), "hi3": np.zeros((n, 3), np.float32),
               "child_begin": np.zeros(n, np.uint32), "child_count": np.zeros(n, np.uint32),
               "prim_begin": np.zeros(n, np.uint32), "prim_count": np.zeros(n, np.uint32),
               "order48": np.zeros((n, 48), np.int8), "depth": np.zeros(n, np.uint32),
               "prim_ids": np.zeros(t, np.uint32)}
        lib().bvhref_export(self._h, *[_p(out[k]) for k in (
            "lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48")],
            16, _p(out["depth"]), _p(out["prim_ids"]))
        out["depth"] = out["depth"].astype(np.uint8)
        out["prim_tri9"] = self.tris[out["prim_ids"]]
        return out

    def trace(self, rays, shadow: bool, *, use_distance: bool = False, packet: int = 0,
              step_cap: int = 0) -> dict:
        """intersectImmediately per ray (packet 0) or intersectWideAlternative
        over packets; rays ``[n, 8]`` = origin, tMax, direction, unused."""
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        out = {"prim": np.zeros(n, np.int32), "t": np.zeros(n, np.float32),
               "pos": np.zeros((n, 3), np.float32), "normal": np.zeros((n, 3), np.float32),
               "occluded": np.zeros(n, np.uint8), "counters": np.zeros((n, 6), np.uint32),
               "depth_hist": np.zeros((2, 64), np.uint64),
               "child_fullness": np.zeros(self.branching + 1, np.uint64),
               "prim_fullness": np.zeros(self.leaf_size + 1, np.uint64)}
        steps = count = None
        if packet and step_cap:
            npk = -(-n // packet)
            steps = out["steps"] = np.zeros((npk, step_cap, 5), np.uint32)
            count = out["step_count"] = np.zeros(npk, np.uint32)
        rc = lib().bvhref_trace(self._h, _p(rays), n, int(shadow), int(use_distance), packet,
                                *[_p(out[k]) for k in ("prim", "t", "pos", "normal", "occluded",
                                                       "counters", "depth_hist")],
                                64, _p(out["child_fullness"]), _p(out["prim_fullness"]),
                                _p(steps), _p(count), step_cap)
        if rc:
            raise RuntimeError(f"reference trace failed ({rc})")
        return out
