"""bvhraytracer_gb300: GB300-native traversal of N-wide BVHs with L-wide leaves.

Host mirror of the reference's trace interface over the C ABI of
libbvhgpu.so (include/bvhgpu.h):

* :class:`Bvh` — the reference's SAH builder (``Bvh`` + ``recursiveBvh``,
  src/accelerationStructure/bvh.cpp:28-40, aabb.cpp:71-206), run on the host
  in C++, with the flat exports of ``CompactNodeManager`` and
  ``FastNodeManager``.
* :class:`Scene` — the flat BVH resident in GPU memory, traced by sm_103a
  kernels.
* :class:`FastNodeManager` / :class:`CompactNodeManager` — batch versions of
  the reference's trace calls (``intersect``, ``intersectSecondary``,
  ``intersectWideAlternative``, ``intersectSecondaryWideAlternative``,
  ``intersectImmediately``) with the reference's semantics per ray.

Rays are ``[n, 8]`` float32 records ``(ox, oy, oz, tmax, dx, dy, dz, pad)``;
closest hits are ``[n, 4]`` records ``(prim as int32 bits, t, u, v)``.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _native as N

__all__ = ["Bvh", "Scene", "FastNodeManager", "CompactNodeManager", "sah_factor", "trace_jobs",
           "camera_rays", "camera_transform", "ao_factor",
           "BvhgpuError", "CLOSEST", "ANY", "PER_RAY", "STREAM", "PERSISTENT", "PROFILE_INSTRUMENTED",
           "PROFILE_FAST"]

BvhgpuError = N.BvhgpuError
CLOSEST, ANY = N.CLOSEST, N.ANY
PER_RAY, STREAM, PERSISTENT = N.PER_RAY, N.STREAM, N.PERSISTENT
PROFILE_INSTRUMENTED, PROFILE_FAST = N.PROFILE_INSTRUMENTED, N.PROFILE_FAST

_KIND = {"closest": N.CLOSEST, "any": N.ANY}
_SCHEME = {"per_ray": N.PER_RAY, "stream": N.STREAM, "persistent": N.PERSISTENT}
_PROFILE = {"instrumented": N.PROFILE_INSTRUMENTED, "fast": N.PROFILE_FAST}
_FORMAT = {"fp32": N.NODES_FP32, "q8": N.NODES_Q8}


def _ptr(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


def sah_factor(branching: int, leaf_size: int, gang: int = 4) -> float:
    """sahNodeFactor of sahFactorConfigSse.txt (RayTracer::loadSahFactor)."""
    out = C.c_float()
    N.check(N.lib().bvhgpu_sah_factor(branching, leaf_size, gang, C.byref(out)))
    return float(out.value)


class Bvh:
    """Host BVH: the reference's SAH build of a triangle soup.

    ``tris``: ``[T, 9]`` (or ``[T, 3, 3]``) float32 world-space points in
    scene-loader order; primitive ids in trace results index this array.
    """

    def __init__(self, tris, branching: int = 4, leaf_size: int = 4, *,
                 leaf_split_option: int = 1, sah: Optional[float] = None, gang: int = 4,
                 sort_each_split: bool = True, drop_zero_area: bool = True):
        t = np.ascontiguousarray(np.asarray(tris, dtype=np.float32).reshape(-1, 9))
        p = N.BuildParams(branching, leaf_size, int(sort_each_split), leaf_split_option,
                          sah_factor(branching, leaf_size, gang) if sah is None else float(sah),
                          int(drop_zero_area))
        h = C.c_void_p()
        N.check(N.lib().bvhgpu_bvh_build(t.ctypes.data, t.shape[0], C.byref(p), C.byref(h)))
        self._adopt(h, p)

    def _adopt(self, h, p) -> None:
        self._h = h
        self.params = p
        info = N.BvhInfo()
        N.check(N.lib().bvhgpu_bvh_info(h, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in N.BvhInfo._fields_}
        self.info["root_lo"] = list(info.root_lo)
        self.info["root_hi"] = list(info.root_hi)

    @classmethod
    def from_compact(cls, arrays: dict, branching: int, leaf_size: int) -> "Bvh":
        """A tree built elsewhere (the reference's own builder), from its
        CompactNodeV3 arrays in the layout :meth:`export_compact` returns
        (bvhgpu_bvh_import_compact)."""
        a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        dt = {"lo3": np.float32, "hi3": np.float32, "child_begin": np.uint32,
              "child_count": np.uint32, "prim_begin": np.uint32, "prim_count": np.uint32,
              "order48": np.int8, "prim_ids": np.uint32, "prim_tri9": np.float32}
        a = {k: np.ascontiguousarray(a[k], dt[k]) for k in dt}
        n = a["child_count"].shape[0]
        h = C.c_void_p()
        N.check(N.lib().bvhgpu_bvh_import_compact(
            n, *[_ptr(a[k]) for k in ("lo3", "hi3", "child_begin", "child_count", "prim_begin",
                                      "prim_count", "order48")],
            a["prim_ids"].shape[0], _ptr(a["prim_ids"]), _ptr(a["prim_tri9"]), branching,
            leaf_size, C.byref(h)))
        self = cls.__new__(cls)
        self._adopt(h, N.BuildParams(branching, leaf_size, 1, 1, 1.0, 1))
        return self

    @property
    def handle(self):
        return self._h

    def export_compact(self) -> dict:
        """CompactNodeV3 view (reference numbering) and sorted primitives."""
        n = self.info["n_nodes"]
        t = self.info["n_tris"]
        out = {
            "lo3": np.zeros((n, 3), np.float32), "hi3": np.zeros((n, 3), np.float32),
            "child_begin": np.zeros(n, np.uint32), "child_count": np.zeros(n, np.uint32),
            "prim_begin": np.zeros(n, np.uint32), "prim_count": np.zeros(n, np.uint32),
            "order48": np.zeros((n, 48), np.int8), "depth": np.zeros(n, np.uint8),
            "prim_ids": np.zeros(t, np.uint32), "prim_tri9": np.zeros((t, 9), np.float32),
        }
        N.check(N.lib().bvhgpu_bvh_export_compact(
            self._h, *[_ptr(out[k]) for k in ("lo3", "hi3", "child_begin", "child_count",
                                              "prim_begin", "prim_count", "order48", "depth",
                                              "prim_ids", "prim_tri9")]))
        return out

    def node_records(self, *, gang: int = 4, leaf_memory: int = 0, node_format: str = "fp32",
                     top_levels: int = 0) -> np.ndarray:
        """Node records of the device layout as encoded on the host (uint8)."""
        p = N.SceneParams(gang, leaf_memory, _FORMAT[node_format], top_levels, 0)
        n = C.c_uint64()
        N.check(N.lib().bvhgpu_bvh_node_records(self._h, C.byref(p), None, 0, C.byref(n)))
        out = np.empty(n.value, np.uint8)
        N.check(N.lib().bvhgpu_bvh_node_records(self._h, C.byref(p), _ptr(out), n.value,
                                                C.byref(n)))
        return out

    def export_fast(self, gang: int = 4, node_memory: int = 0, leaf_memory: int = 0) -> dict:
        """FastNodeManager<gang, node_memory> arrays and trianglePoints."""
        node_memory = node_memory or -(-self.info["branching"] // gang) * gang
        leaf_memory = leaf_memory or -(-self.info["leaf_size"] // gang) * gang
        nn, nf = C.c_uint64(), C.c_uint64()
        N.check(N.lib().bvhgpu_bvh_fast_sizes(self._h, gang, node_memory, leaf_memory,
                                              C.byref(nn), C.byref(nf)))
        n = nn.value
        out = {
            "gang": gang, "node_memory": node_memory, "leaf_memory": leaf_memory,
            "bounds": np.zeros((n, 6 * node_memory), np.float32),
            "begin": np.zeros(n, np.uint32),
            "order": np.zeros((n, 3 * node_memory), np.int8),
            "child_type": np.zeros(n, np.uint32),
            "tri_points": np.zeros(nf.value, np.float32),
        }
        N.check(N.lib().bvhgpu_bvh_export_fast(
            self._h, gang, node_memory, leaf_memory,
            *[_ptr(out[k]) for k in ("bounds", "begin", "order", "child_type", "tri_points")]))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().bvhgpu_bvh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass



def check_noalloc_batch(rays, kind: str, out, device) -> None:
    """Rejects a batch for :meth:`Scene.trace_batches_noalloc` that the kernel
    would read or write out of bounds: rays must be a contiguous float32
    ``[n, 8]`` tensor and ``out`` a contiguous ``[n, 4]`` float32 (closest)
    or ``[n]`` uint8 (any) tensor, both on ``device``. Raises ``ValueError``
    instead of copying, since a copy would allocate."""
    import torch
    if kind not in _KIND:
        raise ValueError(f"no-alloc trace: kind must be 'closest' or 'any', not {kind!r}")
    dev = torch.device(device)
    if not isinstance(rays, torch.Tensor) or not isinstance(out, torch.Tensor):
        raise ValueError("no-alloc trace: rays and out must be tensors")
    for name, t in (("rays", rays), ("out", out)):
        if t.device != dev:
            raise ValueError(f"no-alloc trace: {name} on {t.device}, scene on {dev}")
        if not t.is_contiguous():
            raise ValueError(f"no-alloc trace: {name} must be contiguous (a copy would allocate)")
    if rays.dtype != torch.float32 or rays.dim() != 2 or rays.shape[1] != 8:
        raise ValueError("no-alloc trace: rays must be float32 [n, 8]")
    n = rays.shape[0]
    if _KIND[kind] == N.CLOSEST:
        if out.dtype != torch.float32 or tuple(out.shape) != (n, 4):
            raise ValueError(f"no-alloc trace: closest-hit out must be float32 [{n}, 4]")
    elif out.dtype != torch.uint8 or tuple(out.shape) != (n,):
        raise ValueError(f"no-alloc trace: any-hit out must be uint8 [{n}]")


class Scene:
    """A BVH resident in GPU memory (device layout of the C ABI)."""

    def __init__(self, bvh: Bvh, *, gang: int = 4, leaf_memory: int = 0,
                 node_format: str = "fp32", top_levels: int = 0, device: int = 0):
        p = N.SceneParams(gang, leaf_memory, _FORMAT[node_format], top_levels, device)
        h = C.c_void_p()
        N.check(N.lib().bvhgpu_scene_create(bvh.handle, C.byref(p), C.byref(h)))
        self._h = h
        self.device = device
        self.bvh_info = dict(bvh.info)
        self.node_format = node_format
        b = [C.c_uint64() for _ in range(4)]
        N.check(N.lib().bvhgpu_scene_bytes(h, *[C.byref(x) for x in b]))
        self.node_bytes, self.leaf_bytes, self.node_record_bytes, self.leaf_record_bytes = (
            x.value for x in b)

    @property
    def handle(self):
        return self._h

    def trace(self, rays, *, kind: str = "closest", scheme: str = "per_ray",
              profile: str = "instrumented", workgroup: int = 16, block: int = 128,
              policy: int = 0, refill: int = 0, counters: bool = False,
              depth_hist: bool = False, save_distance: bool = False, reorder: int = 0,
              stack: str = "shared", any_order: bool = False, steps: int = 0,
              wide_alternative: bool = True, out=None, stream=None) -> dict:
        """Traces device rays (torch CUDA tensor ``[n, 8]`` float32).

        Returns ``{"hits": [n,4] f32}`` (closest) or ``{"occluded": [n] u8}``
        (any), plus ``"counters"`` ``[n, 8]`` int32 and ``"depth_hist"``
        ``[2, 64]`` int64 when requested (with ``depth_hist`` also
        ``"fullness"`` ``[2, 17]`` int64: visits of nodes with c children and
        of leaves with c triangles, the reference's Ray::childFullness and
        primitiveFullness summed over the rays). Asynchronous on ``stream``
        (default: torch's current stream). ``save_distance`` (per-ray scheme):
        intersectSaveDistance / intersectImmediately(ray, useDistance=true).
        ``reorder`` = K > 0 traces the rays grouped into 6 K^2 direction bins
        (results identical, in input order). ``stack`` (per-ray scheme):
        ``"shared"`` or ``"local"`` memory for the traversal stacks.
        ``any_order``: any-hit rays without counters push hit children in
        child-index order in both profiles (same results; faster for short
        rays such as ambient occlusion). ``steps`` = S > 0 (stream scheme,
        with ``counters``): also returns ``"step_stats"`` ``[packets, S, 5]``
        (node work, unique nodes, leaf work, unique leaves, terminations per
        step, step 0 the set-up) and ``"step_count"`` ``[packets]``
        (bvhgpu_trace_steps), of intersectWideAlternative's schedule or,
        with ``wide_alternative=False``, intersectWide's.
        """
        import torch
        assert rays.is_cuda and rays.dtype == torch.float32 and rays.shape[-1] == 8
        rays = rays.contiguous()
        n = rays.shape[0]
        k = _KIND[kind]
        res = {}
        dev = rays.device
        if k == N.CLOSEST:
            hits = out if out is not None else torch.empty((n, 4), dtype=torch.float32, device=dev)
            res["hits"] = hits
            hp, op = _ptr(hits), None
        else:
            occ = out if out is not None else torch.empty(n, dtype=torch.uint8, device=dev)
            res["occluded"] = occ
            hp, op = None, _ptr(occ)
        cp = hh = None
        if counters:
            res["counters"] = torch.zeros((n, N.COUNTERS_PER_RAY), dtype=torch.int32, device=dev)
            cp = _ptr(res["counters"])
        if depth_hist:
            hbuf = torch.zeros(2 * 64 + 2 * 17, dtype=torch.int64, device=dev)
            res["depth_hist"] = hbuf[:128].view(2, 64)
            res["fullness"] = hbuf[128:].view(2, 17)
            hh = _ptr(hbuf)
        o = N.TraceOpts(k, _SCHEME[scheme], _PROFILE[profile], workgroup, block, policy, refill,
                        int(save_distance), int(reorder), int(stack == "local"),
                        int(any_order), int(bool(depth_hist)))
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        if steps:
            packets = -(-n // (workgroup * workgroup))
            res["step_stats"] = torch.zeros((packets, steps, 5), dtype=torch.int32, device=dev)
            res["step_count"] = torch.zeros(packets, dtype=torch.int32, device=dev)
            N.check(N.lib().bvhgpu_trace_steps(self._h, _ptr(rays), n, C.byref(o), hp, op, cp, hh,
                                               steps, int(wide_alternative),
                                               _ptr(res["step_stats"]),
                                               _ptr(res["step_count"]),
                                               C.c_void_p(s.cuda_stream)))
            return res
        N.check(N.lib().bvhgpu_trace(self._h, _ptr(rays), n, C.byref(o), hp, op, cp, hh,
                                     C.c_void_p(s.cuda_stream)))
        return res

    def trace_host(self, rays: np.ndarray, *, kind: str = "closest", scheme: str = "per_ray",
                   profile: str = "instrumented", workgroup: int = 16, block: int = 128,
                   policy: int = 0, refill: int = 0, save_distance: bool = False,
                   reorder: int = 0, any_order: bool = False, stack: str = "shared",
                   out: Optional[np.ndarray] = None, stream=None) -> np.ndarray:
        """Host rays in, host results out (copies inside the call); options
        as in :meth:`trace`."""
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        k = _KIND[kind]
        if out is None:
            out = (np.empty((n, 4), np.float32) if k == N.CLOSEST else np.empty(n, np.uint8))
        o = N.TraceOpts(k, _SCHEME[scheme], _PROFILE[profile], workgroup, block, policy, refill,
                        int(save_distance), int(reorder), int(stack == "local"),
                        int(any_order))
        sp = 0
        if stream is not None:
            sp = stream.cuda_stream
        N.check(N.lib().bvhgpu_trace_host(
            self._h, _ptr(rays), n, C.byref(o),
            _ptr(out) if k == N.CLOSEST else None, _ptr(out) if k == N.ANY else None,
            C.c_void_p(sp)))
        return out

    def trace_host_batches(self, batches, *, profile: str = "instrumented", stream=None) -> list:
        """Several host batches in one pipelined call (bvhgpu_trace_host_batches).

        ``batches``: list of ``(rays, kind, out, options)`` with host arrays
        (``out`` may be None) and ``options`` a dict of :meth:`trace`'s
        keyword options (scheme, policy, refill, reorder, any_order, stack,
        block, workgroup). Returns the result arrays, one per batch.
        """
        keep, outs = [], []
        arr = (N.HostBatch * max(1, len(batches)))()
        for i, (rays, kind, out, opt) in enumerate(batches):
            rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
            n = rays.shape[0]
            k = _KIND[kind]
            if out is None:
                out = (np.empty((n, 4), np.float32) if k == N.CLOSEST else np.empty(n, np.uint8))
            opt = dict(opt or {})
            o = N.TraceOpts(k, _SCHEME[opt.get("scheme", "per_ray")], _PROFILE[profile],
                            opt.get("workgroup", 16), opt.get("block", 128),
                            opt.get("policy", 0), opt.get("refill", 0),
                            int(opt.get("save_distance", False)), int(opt.get("reorder", 0)),
                            int(opt.get("stack", "shared") == "local"),
                            int(opt.get("any_order", False)))
            keep += [rays, o]
            arr[i] = N.HostBatch(_ptr(rays), n, C.pointer(o),
                                 _ptr(out) if k == N.CLOSEST else None,
                                 _ptr(out) if k == N.ANY else None)
            outs.append(out)
        sp = stream.cuda_stream if stream is not None else 0
        N.check(N.lib().bvhgpu_trace_host_batches(self._h, arr, len(batches), C.c_void_p(sp)))
        return outs

    def trace_batches_noalloc(self, batches, *, profile: str = "instrumented", policy: int = 0,
                              refill: int = 0, any_order: bool = False, stream=None) -> None:
        """Traces up to 64 batches with no GPU allocation in the call.

        ``batches``: list of ``(rays, kind, out)`` with device tensors: rays
        ``[n, 8]`` float32, kind ``"closest"`` (out ``[n, 4]`` float32) or
        ``"any"`` (out ``[n]`` uint8). For callers that must not allocate GPU
        memory while they trace; the scratch is a fixed array inside the
        library shared by all calls, so calls must not overlap on the GPU.
        """
        import torch
        arr = (N.Batch * max(1, len(batches)))()
        for i, (rays, kind, out) in enumerate(batches):
            check_noalloc_batch(rays, kind, out, self.device)
            k = _KIND[kind]
            arr[i] = N.Batch(_ptr(rays), rays.shape[0], k, 0,
                             _ptr(out) if k == N.CLOSEST else None,
                             _ptr(out) if k == N.ANY else None)
        o = N.TraceOpts(N.CLOSEST, N.PERSISTENT, _PROFILE[profile], 16, 128, policy, refill,
                        0, 0, 0, int(any_order))
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        N.check(N.lib().bvhgpu_trace_batches_noalloc(self._h, arr, len(batches), C.byref(o),
                                                     C.c_void_p(s.cuda_stream)))

    def fp64_check(self, rays, hits, *, profile: str = "instrumented", stream=None):
        """Per closest hit, the FP64 (t, b1, b2) of the same ray / triangle
        pair and |t - t64| / |t64| (``[n, 4]`` float64 tensor; NaN rows for
        misses)."""
        import torch
        n = rays.shape[0]
        out = torch.empty((n, 4), dtype=torch.float64, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device)
        N.check(N.lib().bvhgpu_fp64_check(self._h, _ptr(rays), _ptr(hits), n, _PROFILE[profile],
                                          _ptr(out), C.c_void_p(s.cuda_stream)))
        return out

    def secondary_rays(self, primary, hits, *, light=None, ao_samples: int = 0,
                       ao_length: float = 1.0, sampling: str = "cosine", seed: int = 0,
                       offset: float = 0.001, stream=None):
        """Shadow and AO rays from closest hits on the device
        (bvhgpu_secondary_rays): returns ``(shadow or None, ao or None)``,
        ``[n, 8]`` and ``[n * ao_samples, 8]`` float32 tensors; rays of missed
        primaries are inactive (NaN origin). ``sampling``: ``"cosine"`` or
        ``"reference"`` (the reference's hashed uniform hemisphere, ``seed`` =
        pixel index of primary ray 0)."""
        import torch
        n = primary.shape[0]
        dev = primary.device
        sh = torch.empty((n, 8), dtype=torch.float32, device=dev) if light is not None else None
        ao = (torch.empty((n * ao_samples, 8), dtype=torch.float32, device=dev)
              if ao_samples > 0 else None)
        p = N.Secondary((C.c_float * 3)(*(light if light is not None else (0.0, 0.0, 0.0))),
                        offset, ao_samples, ao_length,
                        N.AO_REFERENCE if sampling == "reference" else N.AO_COSINE, 0, seed)
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        N.check(N.lib().bvhgpu_secondary_rays(self._h, _ptr(primary), _ptr(hits), n, C.byref(p),
                                              _ptr(sh), _ptr(ao), C.c_void_p(s.cuda_stream)))
        return sh, ao

    def set_stack_limit(self, entries: int) -> None:
        """Caps the traversal stack (0 restores the tree's worst case)."""
        N.check(N.lib().bvhgpu_scene_set_stack_limit(self._h, entries))

    def status(self, stream=None) -> None:
        """Raises if a kernel of this scene recorded a device-side error."""
        sp = stream.cuda_stream if stream is not None else 0
        N.check(N.lib().bvhgpu_scene_status(self._h, C.c_void_p(sp)))

    def node_records(self) -> np.ndarray:
        """The device node records, copied to the host (uint8)."""
        n = C.c_uint64()
        N.check(N.lib().bvhgpu_scene_node_records(self._h, None, 0, C.byref(n)))
        out = np.empty(n.value, np.uint8)
        N.check(N.lib().bvhgpu_scene_node_records(self._h, _ptr(out), n.value, C.byref(n)))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().bvhgpu_scene_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def camera_transform(pos, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Camera-to-world matrix, column-major float32, of a camera at ``pos``
    looking at ``target`` (the inverse of a right-handed lookAt: columns
    right, up, -forward, pos)."""
    pos = np.asarray(pos, np.float64)
    f = np.asarray(target, np.float64) - pos
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    m = np.zeros((4, 4), np.float64)  # m[column][row]
    m[0, :3], m[1, :3], m[2, :3], m[3, :3] = r, u, -f, pos
    m[3, 3] = 1.0
    return m.astype(np.float32).reshape(16)


def camera_rays(pos, target, width: int, height: int, *, workgroup: int = 16,
                focal: float = 0.866, tmax: float = 222222.0, transform=None, device: int = 0,
                stream=None):
    """Primary rays on the device (bvhgpu_camera_rays): ``[width * height, 8]``
    float32, tile by tile like CameraFast's workgroups."""
    import torch
    m = camera_transform(pos, target) if transform is None else np.asarray(transform, np.float32)
    cam = N.Camera((C.c_float * 3)(*np.asarray(pos, np.float32)),
                   (C.c_float * 16)(*m.reshape(16)), width, height, workgroup, focal, tmax)
    out = torch.empty((width * height, 8), dtype=torch.float32, device=torch.device("cuda", device))
    s = stream if stream is not None else torch.cuda.current_stream(out.device)
    N.check(N.lib().bvhgpu_camera_rays(C.byref(cam), _ptr(out), C.c_void_p(s.cuda_stream)))
    return out


def ao_factor(occluded, samples: int, stream=None):
    """Per pixel 1 - occluded / samples (bvhgpu_ao_factor), float32."""
    import torch
    n = occluded.shape[0] // samples
    out = torch.empty(n, dtype=torch.float32, device=occluded.device)
    s = stream if stream is not None else torch.cuda.current_stream(occluded.device)
    N.check(N.lib().bvhgpu_ao_factor(_ptr(occluded), n, samples, _ptr(out),
                                     C.c_void_p(s.cuda_stream)))
    return out


def trace_jobs(jobs, *, profile: str = "instrumented", policy: int = 2, refill: int = 16,
               one_launch: bool = False, stream=None) -> None:
    """Traces many (scene, rays) jobs in one persistent launch per ray kind
    (and node width and format), or with ``one_launch`` in a single launch
    whose warps trace one ray kind at a time.

    ``jobs``: list of ``(scene, rays, kind, out)``, ``(scene, rays, kind,
    out, reorder)`` or ``(scene, rays, kind, out, reorder, any_order)`` with
    device tensors (rays ``[n, 8]`` float32; ``out`` ``[n, 4]`` float32 for
    ``"closest"``, ``[n]`` uint8 for ``"any"``); up to 192 jobs, scenes of
    any N, L and node format; ``reorder`` = K groups that job's rays into
    6 K^2 direction bins first; ``any_order`` as in :meth:`Scene.trace`.
    Per-ray results equal
    :meth:`Scene.trace`'s. Stream-ordered (default: torch's current stream)
    and graph-capturable; reordered jobs take stream-ordered scratch.
    """
    import torch
    arr = (N.Job * max(1, len(jobs)))()
    dev = None
    for i, job in enumerate(jobs):
        scene, rays, kind, out = job[:4]
        reorder = job[4] if len(job) > 4 else 0
        any_order = int(job[5]) if len(job) > 5 else 0
        k = _KIND[kind]
        arr[i] = N.Job(scene.handle, _ptr(rays), rays.shape[0], k, reorder,
                       _ptr(out) if k == N.CLOSEST else None, _ptr(out) if k == N.ANY else None,
                       any_order, 0)
        dev = rays.device
    o = N.TraceOpts(N.CLOSEST, N.PERSISTENT, _PROFILE[profile], 16, 128, policy, refill)
    o.one_launch = int(bool(one_launch))
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    N.check(N.lib().bvhgpu_trace_jobs(arr, len(jobs), C.byref(o), C.c_void_p(s.cuda_stream)))


# ---- the reference's ISPC kernels, batched (rayTracerTemplate.ispc) -------

def gang_size() -> int:
    """getGangSize: the fast profile's default gang (4)."""
    return int(N.lib().bvhgpu_gang_size())


def _stream_ptr(t, stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream(t.device)
    return C.c_void_p(s.cuda_stream)


def aabb_intersect(n: int, bounds, offsets, fastrays, distances, stream=None):
    """aabbIntersect{n} for every (offset, FastRay) pair, on device tensors:
    ``bounds`` float32 (node bounds rows of width n), ``offsets`` int32
    ``[count]`` float offsets, ``fastrays`` ``[count, 10]`` float32;
    writes t0 into ``distances`` ``[count, n]`` at hit lanes and returns the
    per-call any-hit flags (uint8)."""
    import torch
    count = offsets.shape[0]
    res = torch.empty(count, dtype=torch.uint8, device=offsets.device)
    N.check(N.lib().bvhgpu_aabb_intersect(n, _ptr(bounds), _ptr(offsets), _ptr(fastrays),
                                          _ptr(distances), _ptr(res), count,
                                          _stream_ptr(offsets, stream)))
    return res


def tri_intersect(l: int, gang: int, tri, tri_ids, fastrays, stream=None):
    """triIntersect{l} for every (leaf offset, FastRay) pair: returns the
    in-leaf index or -1 (int32) and lowers tMax of ``fastrays`` in place."""
    import torch
    count = tri_ids.shape[0]
    res = torch.empty(count, dtype=torch.int32, device=tri_ids.device)
    N.check(N.lib().bvhgpu_tri_intersect(l, gang, _ptr(tri), _ptr(tri_ids), _ptr(fastrays),
                                         _ptr(res), count, _stream_ptr(tri_ids, stream)))
    return res


def tri_any_hit(l: int, tri, tri_ids, fastrays, stream=None):
    """triAnyHit{l} for every (leaf offset, FastRay) pair (uint8)."""
    import torch
    count = tri_ids.shape[0]
    res = torch.empty(count, dtype=torch.uint8, device=tri_ids.device)
    N.check(N.lib().bvhgpu_tri_any_hit(l, _ptr(tri), _ptr(tri_ids), _ptr(fastrays), _ptr(res),
                                       count, _stream_ptr(tri_ids, stream)))
    return res


def read_bandwidth(bytes_: int, *, passes: int = 20, repeats: int = 7, device: int = 0) -> float:
    """Median read bandwidth in GB/s of a ``bytes_`` buffer read ``passes``
    times per timed launch (bvhgpu_read_bandwidth): the L2 ceiling for a
    buffer that fits L2, the HBM read rate for one far larger."""
    g = C.c_double()
    N.check(N.lib().bvhgpu_read_bandwidth(device, int(bytes_), passes, repeats, C.byref(g)))
    return g.value


def hit_prims(hits) -> "np.ndarray":
    """Primitive ids (int32) of a ``[n, 4]`` hit record tensor or array."""
    if isinstance(hits, np.ndarray):
        return hits.view(np.int32)[:, 0]
    return hits.view(dtype=__import__("torch").int32)[:, 0]


class FastNodeManager:
    """Batch form of FastNodeManager's trace calls (fast profile).

    Mirrors fastNodeManager.h: ``intersect`` (1328-1418), ``intersectSecondary``
    (1420-1493), ``intersectWideAlternative`` (835-1049) and
    ``intersectSecondaryWideAlternative`` (1051-1230). Rays use FastRay
    semantics: the direction is used as given (not normalised).
    """

    def __init__(self, bvh: Bvh, leaf_memory: int = 0, *, gang: int = 4,
                 work_group_size: int = 16, node_format: str = "fp32", device: int = 0):
        self.scene = Scene(bvh, gang=gang, leaf_memory=leaf_memory, node_format=node_format,
                           device=device)
        self.work_group_size = work_group_size

    def intersect(self, rays):
        return self.scene.trace(rays, kind="closest", scheme="per_ray", profile="fast")["hits"]

    def intersect_secondary(self, rays):
        return self.scene.trace(rays, kind="any", scheme="per_ray", profile="fast")["occluded"]

    def intersect_wide_alternative(self, rays):
        return self.scene.trace(rays, kind="closest", scheme="stream", profile="fast",
                                workgroup=self.work_group_size)["hits"]

    def intersect_secondary_wide_alternative(self, rays):
        return self.scene.trace(rays, kind="any", scheme="stream", profile="fast",
                                workgroup=self.work_group_size)["occluded"]


class CompactNodeManager:
    """Batch form of CompactNodeManager<CompactNodeV3>'s trace calls with the
    per-ray counters (instrumented profile): ``intersectImmediately``
    (compactNode.cpp:604-814) and ``intersectWideAlternative`` (357-601).
    Directions are normalised like Ray::Ray; t is in world units."""

    def __init__(self, bvh: Bvh, *, gang: int = 4, work_group_size: int = 16, device: int = 0):
        self.scene = Scene(bvh, gang=gang, device=device)
        self.work_group_size = work_group_size

    def intersect_immediately(self, rays, shadow: bool = False, counters: bool = True):
        return self.scene.trace(rays, kind="any" if shadow else "closest", scheme="per_ray",
                                profile="instrumented", counters=counters, depth_hist=counters)

    def intersect_wide_alternative(self, rays, shadow: bool = False, counters: bool = True):
        return self.scene.trace(rays, kind="any" if shadow else "closest", scheme="stream",
                                profile="instrumented", workgroup=self.work_group_size,
                                counters=counters, depth_hist=counters)
