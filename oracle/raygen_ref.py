"""Ray generation restated in numpy float32 — TEST INFRASTRUCTURE ONLY.

Only tests/ use this module, to verify the ray-generation kernels
(bvhgpu_camera_rays, bvhgpu_secondary_rays, bvhgpu_ao_factor). It restates,
operation by operation in float32 (no fused multiply-add), the reference's
arithmetic:

  Camera::getRayTargetPosition ...... src/camera.h:82-98
  FastRay::FastRay .................. src/fastRay.cpp:3-20
  workgroup pixel order ............. src/cameraFast.h:465-490
  getSurfaceNormalPosition .......... src/accelerationStructure/fastNodeManager.h:1700-1713
  computeNormal ..................... src/glmUtil.h:36-39
  secondary origin offset ........... src/cameraFast.h:373, 521
  getAmbientDirection / sampleHemisphere  src/camera.cpp:21-52
  AO factor ......................... src/cameraData.h:403-406

with GLM's published evaluation order (dot = (x*x' + y*y') + z*z', cross,
normalize = v * (1 / sqrt(dot(v, v))), mat4 * vec4 = (m0 x + m1 y) + (m2 z +
m3 w)) and MSVC's std::hash<size_t> = FNV-1a over the value's 8 bytes. GLM is
not vendored and its version is unpinned: parity of this restatement is
unpinned at the reference level. Transcendentals (acos, sin, cos) are numpy's
float32 ones, so directions built from them match the kernels to a few ulps,
not bit for bit.
"""
from __future__ import annotations

import numpy as np

F = np.float32

FNV_OFFSET = 14695981039346656037
FNV_PRIME = 1099511628211


def fnv1a64_bytes(data: bytes) -> int:
    """FNV-1a, 64 bit (Fowler, Noll, Vo)."""
    h = FNV_OFFSET
    for b in data:
        h ^= b
        h = (h * FNV_PRIME) & 0xFFFFFFFFFFFFFFFF
    return h


def fnv1a64_u64(x: int) -> int:
    return fnv1a64_bytes(int(x & 0xFFFFFFFFFFFFFFFF).to_bytes(8, "little"))


def u64_to_f32(x: int) -> np.float32:
    """Round-to-nearest-even conversion of a 64-bit unsigned integer."""
    n = x.bit_length()
    if n <= 24:
        return F(x)
    shift = n - 24
    q, r = x >> shift, x & ((1 << shift) - 1)
    half = 1 << (shift - 1)
    if r > half or (r == half and (q & 1)):
        q += 1
    return F(float(q) * 2.0 ** shift)


def _dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def _cross(x, y):
    return np.stack([x[..., 1] * y[..., 2] - y[..., 1] * x[..., 2],
                     x[..., 2] * y[..., 0] - y[..., 2] * x[..., 0],
                     x[..., 0] * y[..., 1] - y[..., 0] * x[..., 1]], axis=-1)


def _normalize(v):
    return v * (F(1.0) / np.sqrt(_dot(v, v)))[..., None]


def pixel_order(width: int, height: int, tile: int):
    """(row, col) of every emitted ray: tile by tile, row-major inside."""
    ty, tx = -(-height // tile), -(-width // tile)
    rows, cols = [], []
    for a in range(ty):
        for b in range(tx):
            r = np.arange(a * tile, min((a + 1) * tile, height))
            c = np.arange(b * tile, min((b + 1) * tile, width))
            rr, cc = np.meshgrid(r, c, indexing="ij")
            rows.append(rr.reshape(-1))
            cols.append(cc.reshape(-1))
    return np.concatenate(rows), np.concatenate(cols)


def camera_rays(pos, transform, width, height, tile=16, focal=0.866, tmax=222222.0):
    rows, cols = pixel_order(width, height, tile)
    h = -(rows.astype(np.int64) - height // 2)
    w = cols.astype(np.int64) - width // 2
    fh, fw = h.astype(F), w.astype(F)
    inv_w = F(1.0) / F(width)
    z, one = F(0.0), F(1.0)
    ox = (z * fh + one * fw) * inv_w + z
    oy = (one * fh + z * fw) * inv_w + z
    oz = (z * fh + z * fw) * inv_w + (-F(focal))
    ow = (z * fh + z * fw) * inv_w + z
    m = np.asarray(transform, F)
    t = np.stack([(m[0 + k] * ox + m[4 + k] * oy) + (m[8 + k] * oz + m[12 + k] * ow)
                  for k in range(3)], axis=-1)
    p = np.asarray(pos, F)
    target = p[None] + t
    out = np.zeros((rows.shape[0], 8), F)
    out[:, 0:3] = p
    out[:, 3] = F(tmax)
    out[:, 4:7] = target - p[None]
    return out


def _mix64(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def secondary_rays(tris, primary, hits, light=None, offset=0.001, ao_samples=0, ao_length=1.0,
                   sampling="cosine", seed=0):
    """Shadow rays [n, 8] (or None), AO rays [n * ao_samples, 8] (or None) and
    the per-ray normals [n, 3] (NaN for misses)."""
    n = primary.shape[0]
    prim = hits.view(np.int32)[:, 0]
    hit = prim >= 0
    nan_ray = np.array([np.nan, np.nan, np.nan, 0, 1, 1, 1, 0], F)
    tri = np.asarray(tris, F)[np.where(hit, prim, 0)].reshape(n, 3, 3)
    p0, p1, p2 = tri[:, 0], tri[:, 1], tri[:, 2]
    o, d = primary[:, 0:3].astype(F), primary[:, 4:7].astype(F)
    with np.errstate(all="ignore"):
        nrm = _normalize(_cross(p1 - p0, p2 - p0))
        denom = _dot(nrm, d)
        t = _dot(p0 - o, nrm) / denom
        pos = o + d * t[:, None]
        org = pos + nrm * F(offset)
    shadow = None
    if light is not None:
        v = np.asarray(light, F)[None] - org
        dist = np.sqrt(_dot(v, v))
        shadow = np.zeros((n, 8), F)
        shadow[:, 0:3] = org
        shadow[:, 3] = dist
        shadow[:, 4:7] = v * (F(1.0) / dist)[:, None]
        shadow[~hit] = nan_ray
    ao = None
    if ao_samples > 0:
        S = ao_samples
        ao = np.zeros((n, S, 8), F)
        ao[:, :, 0:3] = org[:, None]
        ao[:, :, 3] = F(ao_length)
        if sampling == "reference":
            dirs = np.zeros((n, S, 3), F)
            for i in range(n):
                idx = seed + i
                for k in range(S):
                    u = u64_to_f32(fnv1a64_u64(idx * 599 + k * 223)) / F(2.0 ** 64)
                    v = u64_to_f32(fnv1a64_u64(idx * 181 + k * 691)) / F(2.0 ** 64)
                    phi = np.arccos(F(1.0) - F(2.0) * u)
                    theta = F(2.0 * np.pi * float(v))
                    r = np.array([np.sin(phi) * np.cos(theta), np.sin(phi) * np.sin(theta),
                                  np.cos(phi)], F)
                    if _dot(r, nrm[i]) <= F(0.0):
                        r = -r
                    dirs[i, k] = r
        else:
            ax = np.where((np.abs(nrm[:, 0]) > F(0.9))[:, None], np.array([0, 1, 0], F),
                          np.array([1, 0, 0], F)).astype(F)
            tg = _normalize(_cross(ax, nrm))
            bt = _cross(nrm, tg)
            ids = (np.arange(n, dtype=np.uint64)[:, None] * np.uint64(S)
                   + np.arange(S, dtype=np.uint64)[None])
            h = _mix64(np.uint64(seed) ^ _mix64(ids))
            u1 = (h >> np.uint64(40)).astype(np.uint32).astype(F) * F(1.0 / 16777216.0)
            u2 = (_mix64(h) >> np.uint64(40)).astype(np.uint32).astype(F) * F(1.0 / 16777216.0)
            rr = np.sqrt(u1)
            ph = F(2.0 * np.pi) * u2
            lx, ly = rr * np.cos(ph), rr * np.sin(ph)
            lz = np.sqrt(np.maximum(F(0.0), F(1.0) - u1))
            dirs = (tg[:, None] * lx[..., None] + bt[:, None] * ly[..., None]) + \
                nrm[:, None] * lz[..., None]
        ao[:, :, 4:7] = dirs
        ao[~hit] = nan_ray
        ao = ao.reshape(n * S, 8)
    nrm[~hit] = np.nan
    return shadow, ao, nrm


def ao_factor(occluded, samples):
    c = np.asarray(occluded).reshape(-1, samples).astype(bool).sum(1)
    return (F(1.0) - c.astype(F) / F(samples)).astype(F)
