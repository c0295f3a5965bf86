"""Differentiable closest-hit distance: a torch.autograd.Function over the
C ABI's trace (forward) and adjoint (backward) kernels.

The visibility set is fixed: the forward pass finds each ray's closest
triangle in a BVH built for the current vertex positions, and gradients flow
through the hit triangle's Moller-Trumbore distance and barycentrics (the
formulas of the reference's triIntersect{L}, rayTracerTemplate.ispc:35-76),
not through changes of which triangle is hit. By default the backward kernel
reads the forward pass's stored hits (16 bytes per ray) and runs only the
reverse pass; with ``recompute=True`` it re-traces each ray's hit instead and
nothing is kept between the passes.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import Bvh, Scene
from . import _native as N


class _RayHit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, verts, rays, faces, scene, recompute):
        rc = rays.detach().contiguous()
        res = scene.trace(rc, profile="fast")["hits"]
        ctx.scene = scene
        ctx.n_verts = verts.shape[0]
        ctx.recompute = recompute
        faces32 = faces.to(torch.int32).contiguous()
        if recompute:
            ctx.save_for_backward(rc, faces32)  # the backward re-traces: no hits kept
        else:
            ctx.save_for_backward(rc, faces32, res)
        prim = res.view(torch.int32)[:, 0].clone()
        ctx.mark_non_differentiable(prim)
        return res[:, 1].clone(), res[:, 2].clone(), res[:, 3].clone(), prim

    @staticmethod
    def backward(ctx, gt, gu, gv, _gprim):
        rays, faces = ctx.saved_tensors[:2]
        n = rays.shape[0]
        dev = rays.device

        def g(x):
            # incoming gradient of t, u or v as a contiguous float32 array (None: zero)
            return None if x is None else x.to(torch.float32).contiguous()

        gt, gu, gv = g(gt), g(gu), g(gv)
        grad_rays = torch.empty((n, 8), dtype=torch.float32, device=dev)
        grad_verts = torch.zeros((ctx.n_verts, 3), dtype=torch.float32, device=dev)
        stream = torch.cuda.current_stream(dev)
        # The kernels add each hit triangle's vertex gradients straight into
        # grad_verts through the face indices.
        if ctx.recompute:
            # Re-trace each ray's closest hit (the same fast-profile traversal
            # as the forward pass, so the same triangle), with the incoming
            # gradients as (unused, dL/dt, dL/du, dL/dv) records.
            z = torch.zeros(n, dtype=torch.float32, device=dev)
            grad_hits = torch.stack([z] + [z if x is None else x for x in (gt, gu, gv)],
                                    dim=1).contiguous()
            N.check(N.lib().bvhgpu_adjoint_vertices(
                ctx.scene.handle, rays.data_ptr(), n, grad_hits.data_ptr(), faces.data_ptr(),
                faces.shape[0], ctx.n_verts, grad_verts.data_ptr(), grad_rays.data_ptr(),
                C.c_void_p(stream.cuda_stream)))
        else:
            hits = ctx.saved_tensors[2]
            N.check(N.lib().bvhgpu_adjoint_hits(
                ctx.scene.handle, rays.data_ptr(), hits.data_ptr(), n,
                *[None if x is None else x.data_ptr() for x in (gt, gu, gv)],
                faces.data_ptr(), faces.shape[0], ctx.n_verts, grad_verts.data_ptr(), None,
                grad_rays.data_ptr(), C.c_void_p(stream.cuda_stream)))
        return grad_verts, grad_rays, None, None, None


def ray_hit(verts: torch.Tensor, faces: torch.Tensor, rays: torch.Tensor, scene: Scene,
            recompute: bool = False):
    """Closest hit of each ray: returns ``(t, u, v, prim)``; ``t``, ``u``, ``v``
    are differentiable with respect to ``verts`` ``[V, 3]`` and ``rays``
    ``[n, 8]`` (origin and direction). ``scene`` must be built from
    ``verts[faces]`` (see :func:`scene_for`). Misses have prim -1, t = tmax and
    zero gradients.

    ``recompute=False`` keeps the forward pass's hit records (16 bytes per
    ray) for the backward pass, which then runs no traversal;
    ``recompute=True`` keeps none and the backward pass re-traces each ray
    (FP32 node scenes only). Both give the same per-ray gradients; the vertex
    gradients differ only in the order of their atomic sums."""
    return _RayHit.apply(verts, rays, faces, scene, bool(recompute))


def scene_for(verts: torch.Tensor, faces: torch.Tensor, branching: int = 8, leaf_size: int = 8,
              device: int = 0) -> Scene:
    """BVH and device scene of the mesh at its current vertex positions."""
    tris = verts.detach().cpu()[faces.cpu()].reshape(-1, 9).numpy()
    return Scene(Bvh(tris, branching, leaf_size, drop_zero_area=False), device=device)


def moller_trumbore_torch(o, d, p0, p1, p2):
    """Plain PyTorch Moller-Trumbore (t, b1, b2) of given ray/triangle pairs,
    in the order of triIntersect{L}; differentiable by autograd."""
    e1 = p1 - p0
    e2 = p2 - p0
    s1 = torch.cross(d, e2, dim=-1)
    div = (s1 * e1).sum(-1)
    inv = 1.0 / div
    s = o - p0
    b1 = (s * s1).sum(-1) * inv
    s2 = torch.cross(s, e1, dim=-1)
    b2 = (d * s2).sum(-1) * inv
    t = (e2 * s2).sum(-1) * inv
    return t, b1, b2
