"""Seeded synthetic scenes and ray batches (numpy, float32).

The reference measured on glTF scenes that are not available here; these
generators stand in for them with the sizes and value distributions of the
benchmark configurations:

* :func:`terrain` — height field on an ``n x n`` quad grid over [0,1]^2
  (x, z), height y = sum of 4 sine octaves (frequencies 1, 2, 4, 8,
  amplitude 0.1/k, seeded phases and directions). ``n=128`` gives 32,768
  triangles.
* :func:`clutter` — ``n_objects`` UV spheres (16 x 8: 256 triangles) and
  boxes subdivided 4 x 4 per face (192 triangles) in a 20 x 4 x 10 room
  (x, y-up, z) whose six walls are 8 x 8 grids; sizes log-uniform in
  [0.05, 1], centres in 30 Gaussian blobs (sigma 1). The room, the blob
  count and sigma scale with ``n_objects / 4000`` (cube root for lengths).

Convention: y is up, as in the reference camera (lookAt up = (0, 1, 0),
src/camera.h:48-58). Triangles are returned as ``[T, 9]`` float32 arrays in
loader order.

Ray records are ``[n, 8]`` float32: ``(ox, oy, oz, tmax, dx, dy, dz, 0)``.
"""
from __future__ import annotations

import math

import numpy as np

FOCAL_60 = 0.866  # Camera focal length for a 60 degree horizontal FOV (camera.h:44-49)
DEFAULT_TMAX = 222222.0  # FastRay / Ray default tMax (fastRay.h:27, ray.cpp:30)


# --------------------------------------------------------------- geometry --
def _grid_tris(verts: np.ndarray) -> np.ndarray:
    """Triangles of a (m+1) x (n+1) vertex grid, two per quad."""
    a = verts[:-1, :-1]
    b = verts[1:, :-1]
    c = verts[1:, 1:]
    d = verts[:-1, 1:]
    t1 = np.stack([a, c, b], axis=2)
    t2 = np.stack([a, d, c], axis=2)
    return np.stack([t1, t2], axis=2).reshape(-1, 9).astype(np.float32)


def _terrain_grid(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, n + 1)
    x, z = np.meshgrid(xs, xs, indexing="ij")
    y = np.zeros_like(x)
    for k, f in enumerate((1, 2, 4, 8), start=1):
        th = rng.uniform(0, 2 * math.pi)
        ph = rng.uniform(0, 2 * math.pi)
        y += (0.1 / k) * np.sin(2 * math.pi * f * (x * math.cos(th) + z * math.sin(th)) + ph)
    return np.stack([x, y, z], axis=-1)


def terrain(n: int = 128, seed: int = 0) -> np.ndarray:
    """Height-field terrain with ``2*n*n`` triangles."""
    return _grid_tris(_terrain_grid(n, seed))


def terrain_mesh(n: int = 128, seed: int = 0):
    """The same terrain as shared vertices ``[(n+1)^2, 3]`` float32 and faces
    ``[2 n^2, 3]`` int64, in the triangle order of :func:`terrain`."""
    verts = _terrain_grid(n, seed).reshape(-1, 3).astype(np.float32)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = i * (n + 1) + j
    b = (i + 1) * (n + 1) + j
    c = (i + 1) * (n + 1) + j + 1
    d = i * (n + 1) + j + 1
    t1 = np.stack([a, c, b], -1)
    t2 = np.stack([a, d, c], -1)
    faces = np.stack([t1, t2], axis=2).reshape(-1, 3).astype(np.int64)
    return verts, faces


def _uv_sphere(center, radius, seg: int = 16, rings: int = 8) -> np.ndarray:
    """UV sphere: ``seg`` longitudes, ``rings`` vertex rings between the poles."""
    th = np.linspace(0, math.pi, rings + 2)[1:-1]
    ph = np.linspace(0, 2 * math.pi, seg + 1)[:-1]
    ring = np.stack([np.sin(th)[:, None] * np.cos(ph)[None, :],
                     np.repeat(np.cos(th)[:, None], seg, 1),
                     np.sin(th)[:, None] * np.sin(ph)[None, :]], axis=-1)
    ring = center + radius * ring  # [rings, seg, 3]
    top = center + np.array([0, radius, 0])
    bot = center - np.array([0, radius, 0])
    tris = []
    j = np.arange(seg)
    jn = (j + 1) % seg
    tris.append(np.stack([np.broadcast_to(top, (seg, 3)), ring[0, jn], ring[0, j]], 1))
    for r in range(rings - 1):
        a, b = ring[r, j], ring[r, jn]
        c, d = ring[r + 1, jn], ring[r + 1, j]
        tris.append(np.stack([a, b, c], 1))
        tris.append(np.stack([a, c, d], 1))
    tris.append(np.stack([np.broadcast_to(bot, (seg, 3)), ring[-1, j], ring[-1, jn]], 1))
    return np.concatenate(tris).reshape(-1, 9)


def _box(center, half, sub: int = 4, outward: bool = True) -> np.ndarray:
    """Axis-aligned box with each face subdivided ``sub x sub``; faces wound
    so their geometric normals point out of the box (or into it)."""
    s = np.linspace(-1.0, 1.0, sub + 1)
    u, v = np.meshgrid(s, s, indexing="ij")
    faces = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            p = np.zeros(u.shape + (3,))
            a1, a2 = (axis + 1) % 3, (axis + 2) % 3
            p[..., axis] = sign
            if sign > 0:
                p[..., a1], p[..., a2] = u, v
            else:
                p[..., a1], p[..., a2] = v, u
            faces.append(_grid_tris(center + half * p))
    tris = np.concatenate(faces)
    if outward:  # swap p1 and p2 to flip the winding
        tris = tris.reshape(-1, 3, 3)[:, [0, 2, 1]].reshape(-1, 9)
    return tris


def clutter_objects(n_objects: int = 4000, seed: int = 1, sphere_fraction: float = 0.9,
                    blobs: int = 30):
    """Object placement of :func:`clutter`: (room, centres, sizes, is_sphere, aspect)."""
    rng = np.random.default_rng(seed)
    scale = (n_objects / 4000.0) ** (1.0 / 3.0)
    room = np.array([20.0, 4.0, 10.0]) * scale
    n_blobs = max(1, int(round(blobs * n_objects / 4000.0)))
    centers = rng.uniform(room * 0.05, room * 0.95, size=(n_blobs, 3))
    which = rng.integers(0, n_blobs, n_objects)
    pos = centers[which] + rng.normal(0.0, 1.0 * scale, (n_objects, 3))
    pos = np.clip(pos, room * 0.01, room * 0.99)
    size = np.exp(rng.uniform(math.log(0.05), math.log(1.0), n_objects))
    is_sphere = rng.uniform(size=n_objects) < sphere_fraction
    aspect = rng.uniform(0.5, 1.0, (n_objects, 3))
    return room, pos, size, is_sphere, aspect


def clutter(n_objects: int = 4000, seed: int = 1, sphere_fraction: float = 0.9,
            blobs: int = 30) -> np.ndarray:
    """Cluttered room; about 250 triangles per object."""
    room, pos, size, is_sphere, aspect = clutter_objects(n_objects, seed, sphere_fraction, blobs)
    parts = []
    # Room walls (floor, ceiling, four walls), 8 x 8 quads each, facing inward.
    parts.append(_box(room / 2, room / 2, sub=8, outward=False))
    for i in range(n_objects):
        if is_sphere[i]:
            parts.append(_uv_sphere(pos[i], size[i] / 2))
        else:
            parts.append(_box(pos[i], size[i] / 2 * aspect[i]))
    return np.concatenate(parts).astype(np.float32)


def _clearest(candidates: np.ndarray, pos: np.ndarray, size: np.ndarray) -> np.ndarray:
    """The candidate point farthest from every object's bounding sphere."""
    best, best_c = -np.inf, candidates[0]
    for c in candidates:
        clear = np.min(np.linalg.norm(pos - c, axis=1) - size * 0.5 * math.sqrt(3.0))
        if clear > best:
            best, best_c = clear, c
    return best_c


def clutter_viewpoints(n_objects: int = 4000, seed: int = 1):
    """Camera position, camera target and point-light position for the
    clutter scene, placed in free space (largest clearance to any object):
    the camera near the x = 0 wall at mid height looking down the room, the
    light under the ceiling near the room centre."""
    room, pos, size, _, _ = clutter_objects(n_objects, seed)
    g = np.stack(np.meshgrid(np.linspace(0.03, 0.2, 6), np.linspace(0.35, 0.65, 5),
                             np.linspace(0.3, 0.7, 9), indexing="ij"), -1).reshape(-1, 3)
    cam = _clearest(g * room, pos, size)
    target = np.array([0.95, 0.4, 0.5]) * room
    gl = np.stack(np.meshgrid(np.linspace(0.35, 0.65, 7), np.linspace(0.8, 0.95, 4),
                              np.linspace(0.3, 0.7, 7), indexing="ij"), -1).reshape(-1, 3)
    light = _clearest(gl * room, pos, size)
    return cam, target, light.astype(np.float32)


def scene_diagonal(tris: np.ndarray) -> float:
    p = tris.reshape(-1, 3)
    return float(np.linalg.norm(p.max(0) - p.min(0)))


# ------------------------------------------------------------------- rays --
def _normalize(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def camera_rays(pos, target, width: int, height: int, *, tile: int = 16,
                focal: float = FOCAL_60, tmax: float = DEFAULT_TMAX) -> np.ndarray:
    """Pinhole primary rays like Camera::getRayTargetPosition (camera.h:82-98).

    Pixel (w, h) with w in [-W/2, W/2), h in (H/2 .. -H/2] maps to the target
    ``pos + R (w/W, h/W, -focal)`` with R the inverse lookAt rotation
    (up = +y); the direction is target - pos, not normalised (FastRay). Rays
    are emitted tile by tile (``tile x tile`` pixels, row-major inside a
    tile) like the reference's workgroups; partial edge tiles are included.
    """
    pos = np.asarray(pos, np.float64)
    f = _normalize(np.asarray(target, np.float64) - pos)
    r = _normalize(np.cross(f, [0.0, 1.0, 0.0]))
    u = np.cross(r, f)
    ty, tx = -(-height // tile), -(-width // tile)
    jj, ii = np.meshgrid(np.arange(tile), np.arange(tile), indexing="ij")  # row, col in tile
    rows = (np.arange(ty)[:, None, None, None] * tile + jj[None, None]).astype(np.int64)
    cols = (np.arange(tx)[None, :, None, None] * tile + ii[None, None]).astype(np.int64)
    rows, cols = np.broadcast_arrays(rows, cols)
    keep = (rows < height) & (cols < width)
    rows, cols = rows[keep], cols[keep]
    w = cols - width / 2.0
    h = -(rows - height / 2.0)
    d = (r[None] * (w / width)[:, None] + u[None] * (h / width)[:, None] + f[None] * focal)
    out = np.zeros((d.shape[0], 8), np.float32)
    out[:, 0:3] = pos
    out[:, 3] = tmax
    out[:, 4:7] = d
    return out


def surface(tris: np.ndarray, rays: np.ndarray, prims: np.ndarray):
    """Hit position and geometric normal like getSurfaceNormalPosition
    (fastNodeManager.h:1700-1713): n = normalize(cross(p1-p0, p2-p0)), the
    point from the ray-plane intersection. Returns (hit_mask, pos, normal)."""
    m = prims >= 0
    t = tris[prims[m]].reshape(-1, 3, 3).astype(np.float32)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    n = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
    o = rays[m, 0:3]
    d = rays[m, 4:7]
    denom = np.sum(n * d, axis=1)
    tt = np.sum((t[:, 0] - o) * n, axis=1) / denom
    p = (o + d * tt[:, None]).astype(np.float32)
    return m, p, n


def shadow_rays(pos: np.ndarray, normal: np.ndarray, light, offset: float = 0.001) -> np.ndarray:
    """One shadow ray per hit toward a point light; unit direction, tmax =
    distance to the light; origin offset along the normal (cameraFast.h:373)."""
    o = pos + normal * offset
    v = np.asarray(light, np.float32)[None] - o
    dist = np.linalg.norm(v, axis=1)
    out = np.zeros((o.shape[0], 8), np.float32)
    out[:, 0:3] = o
    out[:, 3] = dist
    out[:, 4:7] = v / dist[:, None]
    return out


def ao_rays(pos: np.ndarray, normal: np.ndarray, samples: int, length: float, seed: int = 7,
            offset: float = 0.001) -> np.ndarray:
    """``samples`` cosine-distributed ambient-occlusion rays per hit, unit
    direction, tmax = ``length``; sample-major order inside each hit."""
    rng = np.random.default_rng(seed)
    nh = pos.shape[0]
    u1 = rng.random((nh, samples))
    u2 = rng.random((nh, samples))
    rr = np.sqrt(u1)
    phi = 2 * math.pi * u2
    lx, ly, lz = rr * np.cos(phi), rr * np.sin(phi), np.sqrt(np.maximum(0.0, 1 - u1))
    n = normal.astype(np.float64)
    a = np.where(np.abs(n[:, :1]) > 0.9, [[0.0, 1.0, 0.0]], [[1.0, 0.0, 0.0]])
    t = _normalize(np.cross(a, n))
    b = np.cross(n, t)
    d = (t[:, None] * lx[..., None] + b[:, None] * ly[..., None] + n[:, None] * lz[..., None])
    out = np.zeros((nh, samples, 8), np.float32)
    out[..., 0:3] = (pos + normal * offset)[:, None]
    out[..., 3] = length
    out[..., 4:7] = d
    return out.reshape(-1, 8)


def terrain_workload(n: int = 128, res: int = 512, seed: int = 0):
    """Terrain triangles and 512 x 512 primary rays from a camera 1.5 above
    the terrain plane looking at its centre pitched 45 degrees down (so the
    view covers the terrain), 60 degree FOV; light at (2, 3, 2)."""
    tris = terrain(n, seed)
    centre = np.array([0.5, 0.0, 0.5])
    pos = centre + np.array([0.0, 1.5, 1.5])
    rays = camera_rays(pos, centre, res, res)
    return tris, rays, np.array([2.0, 3.0, 2.0], np.float32)


def clutter_camera(n_objects: int = 4000, width: int = 1920, height: int = 1080, seed: int = 1):
    """Primary rays of the clutter scene from :func:`clutter_viewpoints`."""
    cam, target, _ = clutter_viewpoints(n_objects, seed)
    return camera_rays(cam, target, width, height)
