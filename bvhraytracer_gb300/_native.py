"""ctypes binding of libbvhgpu.so (the C ABI declared in include/bvhgpu.h).

The library is built in-tree by ``bvhraytracer_gb300.build``. Loading fails
loudly when it is missing: there is no CPU fallback for any traced call.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import os

# BVHGPU_LIBRARY may point at another build of the same library (tuning runs).
LIB_PATH = Path(os.environ.get("BVHGPU_LIBRARY",
                               Path(__file__).resolve().parent / "_build" / "libbvhgpu.so"))

OK = 0
ERR_BAD_ARG = 1
ERR_OOM = 2
ERR_CUDA = 3
ERR_STACK_OVERFLOW = 4
ERR_TIMEOUT = 5
ERR_UNSUPPORTED = 6
ERR_NO_DEVICE = 7

CLOSEST, ANY = 0, 1
PER_RAY, STREAM, PERSISTENT = 0, 1, 2
PROFILE_INSTRUMENTED, PROFILE_FAST = 0, 1
NODES_FP32, NODES_Q8 = 0, 1
COUNTERS_PER_RAY = 8


class BuildParams(C.Structure):
    _fields_ = [("branching", C.c_int32), ("leaf_size", C.c_int32),
                ("sort_each_split", C.c_int32), ("leaf_split_option", C.c_int32),
                ("sah_factor", C.c_float), ("drop_zero_area", C.c_int32)]


class BvhInfo(C.Structure):
    _fields_ = [("n_input_tris", C.c_uint64), ("n_tris", C.c_uint64), ("n_nodes", C.c_uint64),
                ("n_inner", C.c_uint64), ("n_leaves", C.c_uint64), ("depth", C.c_int32),
                ("max_stack", C.c_int32), ("branching", C.c_int32), ("leaf_size", C.c_int32),
                ("root_lo", C.c_float * 3), ("root_hi", C.c_float * 3)]


class SceneParams(C.Structure):
    _fields_ = [("gang", C.c_int32), ("leaf_memory", C.c_int32), ("node_format", C.c_int32),
                ("top_levels", C.c_int32), ("device", C.c_int32)]


class TraceOpts(C.Structure):
    _fields_ = [("kind", C.c_int32), ("scheme", C.c_int32), ("profile", C.c_int32),
                ("workgroup", C.c_int32), ("block", C.c_int32), ("policy", C.c_int32),
                ("refill", C.c_int32), ("save_distance", C.c_int32),
                ("reorder", C.c_int32), ("stack_local", C.c_int32), ("any_order", C.c_int32),
                ("fullness", C.c_int32), ("one_launch", C.c_int32)]


class Batch(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("n", C.c_uint64), ("kind", C.c_int32), ("pad", C.c_int32),
                ("hits", C.c_void_p), ("occluded", C.c_void_p)]


class HostBatch(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("n", C.c_uint64), ("opts", C.POINTER(TraceOpts)),
                ("hits", C.c_void_p), ("occluded", C.c_void_p)]


class Job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("rays", C.c_void_p), ("n", C.c_uint64),
                ("kind", C.c_int32), ("reorder", C.c_int32), ("hits", C.c_void_p),
                ("occluded", C.c_void_p), ("any_order", C.c_int32), ("pad", C.c_int32)]


MAX_JOBS = 192


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("transform", C.c_float * 16), ("width", C.c_uint32),
                ("height", C.c_uint32), ("workgroup", C.c_int32), ("focal", C.c_float),
                ("tmax", C.c_float)]


class Secondary(C.Structure):
    _fields_ = [("light", C.c_float * 3), ("offset", C.c_float), ("ao_samples", C.c_int32),
                ("ao_length", C.c_float), ("sampling", C.c_int32), ("pad", C.c_int32),
                ("seed", C.c_uint64)]


AO_COSINE, AO_REFERENCE = 0, 1


class BvhgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"bvhgpu error {code}: {msg}")
        self.code = code


_lib = None
_lock = threading.Lock()

_P = C.c_void_p
_SIGS = {
    "bvhgpu_last_error": (C.c_char_p, []),
    "bvhgpu_bvh_build": (C.c_int, [_P, C.c_uint64, C.POINTER(BuildParams), C.POINTER(_P)]),
    "bvhgpu_bvh_info": (C.c_int, [_P, C.POINTER(BvhInfo)]),
    "bvhgpu_bvh_import_compact": (C.c_int, [C.c_uint64] + [_P] * 7 + [C.c_uint64, _P, _P,
                                            C.c_int32, C.c_int32, C.POINTER(_P)]),
    "bvhgpu_bvh_free": (C.c_int, [_P]),
    "bvhgpu_sah_factor": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
    "bvhgpu_bvh_export_compact": (C.c_int, [_P] + [_P] * 10),
    "bvhgpu_bvh_fast_sizes": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32,
                                        C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "bvhgpu_bvh_export_fast": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32] + [_P] * 5),
    "bvhgpu_scene_create": (C.c_int, [_P, C.POINTER(SceneParams), C.POINTER(_P)]),
    "bvhgpu_scene_free": (C.c_int, [_P]),
    "bvhgpu_scene_bytes": (C.c_int, [_P] + [C.POINTER(C.c_uint64)] * 4),
    "bvhgpu_trace": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(TraceOpts), _P, _P, _P, _P, _P]),
    "bvhgpu_trace_host": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(TraceOpts), _P, _P, _P]),
    "bvhgpu_fp64_check": (C.c_int, [_P, _P, _P, C.c_uint64, C.c_int32, _P, _P]),
    "bvhgpu_read_bandwidth": (C.c_int, [C.c_int32, C.c_uint64, C.c_int32, C.c_int32,
                                        C.POINTER(C.c_double)]),
    "bvhgpu_scene_set_stack_limit": (C.c_int, [_P, C.c_int32]),
    "bvhgpu_scene_inject_stall": (C.c_int, [_P, C.c_int32]),
    "bvhgpu_adjoint": (C.c_int, [_P, _P, C.c_uint64, _P, _P, _P, _P]),
    "bvhgpu_adjoint_vertices": (C.c_int, [_P, _P, C.c_uint64, _P, _P, C.c_uint64, C.c_uint64,
                                          _P, _P, _P]),
    "bvhgpu_adjoint_hits": (C.c_int, [_P, _P, _P, C.c_uint64, _P, _P, _P, _P, C.c_uint64,
                                      C.c_uint64, _P, _P, _P, _P]),
    "bvhgpu_trace_jobs": (C.c_int, [C.POINTER(Job), C.c_int32, C.POINTER(TraceOpts), _P]),
    "bvhgpu_trace_host_batches": (C.c_int, [_P, C.POINTER(HostBatch), C.c_int32, _P]),
    "bvhgpu_gang_size": (C.c_int, []),
    "bvhgpu_trace_steps": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(TraceOpts), _P, _P, _P, _P,
                                     C.c_int32, C.c_int32, _P, _P, _P]),
    "bvhgpu_aabb_intersect": (C.c_int, [C.c_int32, _P, _P, _P, _P, _P, C.c_uint64, _P]),
    "bvhgpu_tri_intersect": (C.c_int, [C.c_int32, C.c_int32, _P, _P, _P, _P, C.c_uint64, _P]),
    "bvhgpu_tri_any_hit": (C.c_int, [C.c_int32, _P, _P, _P, _P, C.c_uint64, _P]),
    "bvhgpu_intersect_fastrays": (C.c_int, [_P, _P, C.c_uint64, C.c_int32, _P, _P, _P]),
    "bvhgpu_intersect_secondary_fastrays": (C.c_int, [_P, _P, C.c_uint64, C.c_int32, _P, _P]),
    "bvhgpu_trace_batches_noalloc": (C.c_int, [_P, C.POINTER(Batch), C.c_int32,
                                                C.POINTER(TraceOpts), _P]),
    "bvhgpu_scene_status": (C.c_int, [_P, _P]),
    "bvhgpu_camera_rays": (C.c_int, [C.POINTER(Camera), _P, _P]),
    "bvhgpu_secondary_rays": (C.c_int, [_P, _P, _P, C.c_uint64, C.POINTER(Secondary), _P, _P,
                                        _P]),
    "bvhgpu_ao_factor": (C.c_int, [_P, C.c_uint64, C.c_int32, _P, _P]),
    "bvhgpu_scene_node_records": (C.c_int, [_P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "bvhgpu_bvh_node_records": (C.c_int, [_P, C.POINTER(SceneParams), _P, C.c_uint64,
                                          C.POINTER(C.c_uint64)]),
}

# Every symbol the public header declares (checked by the CPU tests).
EXPORTED = tuple(_SIGS)


def lib() -> C.CDLL:
    """Loads libbvhgpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with bvhraytracer_gb300.build.build()")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != OK:
        msg = lib().bvhgpu_last_error()
        raise BvhgpuError(rc, msg.decode() if msg else "")
