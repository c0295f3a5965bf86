"""glTF 2.0 scene input and output for the triangle soup the builder takes.

:func:`load_gltf` restates the reference's loading path: ``loadGltfModel``
(src/modelLoader.h:23-341) reads every mesh primitive's POSITION accessor and
index accessor (unsigned int / short / byte), every node becomes a game object
with its children, nodes without a parent hang under the root in node order
(src/rayTracer.cpp:491-509), global transforms are parent * translate *
rotate * scale (gameobject.h:58-79), and ``GameObject::iterateGo``
(gameobject.h:110-146) emits each object's triangles mesh by mesh, index
triple by index triple, then its children's, skipping triangles of zero
surface area. Vertex positions are transformed in float32 like
``Triangle::updatePoints`` (triangle.cpp:26-39).

:func:`write_gltf` writes a mesh in the subset that loader reads (POSITION,
NORMAL and TEXCOORD_0 accessors, 32-bit indices, one material with a white
base colour), so the synthetic scenes can be opened by the reference.

Transforms use GLM's published formulas (mat4_cast of a unit quaternion,
column-major matrices, mat4 * mat4 column by column, mat4 * vec4 as
(m0 x + m1 y) + (m2 z + m3 w)); GLM is
not vendored and its version is unpinned, so node transforms other than the
identity are not bit-for-bit pinned to the reference.
"""
from __future__ import annotations

import base64
import json
import struct
from pathlib import Path

import numpy as np

F = np.float32
_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32,
              5126: np.float32}
_GLB_MAGIC, _CHUNK_JSON, _CHUNK_BIN = 0x46546C67, 0x4E4F534A, 0x004E4942


def _read_container(path: Path):
    data = path.read_bytes()
    if path.suffix.lower() == ".glb":
        magic, _version, _length = struct.unpack_from("<III", data, 0)
        if magic != _GLB_MAGIC:
            raise ValueError(f"{path}: not a binary glTF file")
        off, doc, binary = 12, None, None
        while off < len(data):
            clen, ctype = struct.unpack_from("<II", data, off)
            chunk = data[off + 8:off + 8 + clen]
            if ctype == _CHUNK_JSON:
                doc = json.loads(chunk.decode("utf-8"))
            elif ctype == _CHUNK_BIN:
                binary = chunk
            off += 8 + clen
        if doc is None:
            raise ValueError(f"{path}: no JSON chunk")
        return doc, binary
    return json.loads(data.decode("utf-8")), None


def _buffers(doc, path: Path, binary):
    out = []
    for i, b in enumerate(doc.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            if binary is None or i != 0:
                raise ValueError("buffer without uri outside a .glb file")
            out.append(binary)
        elif uri.startswith("data:"):
            out.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            out.append((path.parent / uri).read_bytes())
    return out


def _accessor(doc, bufs, idx: int, ncomp: int) -> np.ndarray:
    """Tightly packed accessor data, as the reference reads it (it casts the
    buffer to glm::vec3 / integer arrays and ignores byteStride)."""
    acc = doc["accessors"][idx]
    view = doc["bufferViews"][acc["bufferView"]]
    dt = _COMPONENT[acc["componentType"]]
    start = view.get("byteOffset", 0) + acc.get("byteOffset", 0)
    count = acc["count"] * ncomp
    raw = bufs[view["buffer"]]
    return np.frombuffer(raw, dt, count, start).reshape(acc["count"], ncomp) if ncomp > 1 else \
        np.frombuffer(raw, dt, count, start)


def _quat_mat(q) -> np.ndarray:
    """glm::mat4_cast of (x, y, z, w), column-major [col][row], float32."""
    x, y, z, w = (F(v) for v in q)
    qxx, qyy, qzz = x * x, y * y, z * z
    qxz, qxy, qyz = x * z, x * y, y * z
    qwx, qwy, qwz = w * x, w * y, w * z
    one, two = F(1), F(2)
    m = np.eye(4, dtype=F)
    m[0, 0] = one - two * (qyy + qzz)
    m[0, 1] = two * (qxy + qwz)
    m[0, 2] = two * (qxz - qwy)
    m[1, 0] = two * (qxy - qwz)
    m[1, 1] = one - two * (qxx + qzz)
    m[1, 2] = two * (qyz + qwx)
    m[2, 0] = two * (qxz + qwy)
    m[2, 1] = two * (qyz - qwx)
    m[2, 2] = one - two * (qxx + qyy)
    return m


def _mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Column-major mat4 product a * b, GLM's evaluation: column c of the
    result is ((a0 b[c][0] + a1 b[c][1]) + a2 b[c][2]) + a3 b[c][3]."""
    out = np.zeros((4, 4), F)
    for c in range(4):
        out[c] = ((a[0] * b[c, 0] + a[1] * b[c, 1]) + a[2] * b[c, 2]) + a[3] * b[c, 3]
    return out


def _local(node) -> np.ndarray:
    if "matrix" in node:
        return np.asarray(node["matrix"], F).reshape(4, 4)  # column-major already
    t = np.eye(4, dtype=F)
    t[3, :3] = np.asarray(node.get("translation", (0, 0, 0)), F)
    r = _quat_mat(node.get("rotation", (0, 0, 0, 1)))
    s = np.eye(4, dtype=F)
    sc = np.asarray(node.get("scale", (1, 1, 1)), F)
    s[0, 0], s[1, 1], s[2, 2] = sc
    return _mul(_mul(t, r), s)


def _transform(m: np.ndarray, p: np.ndarray) -> np.ndarray:
    one = F(1)
    return ((m[0][None, :3] * p[:, 0:1] + m[1][None, :3] * p[:, 1:2])
            + (m[2][None, :3] * p[:, 2:3] + m[3][None, :3] * one)).astype(F)


def _nonzero_area(tri: np.ndarray) -> np.ndarray:
    a = tri[:, 1] - tri[:, 0]
    b = tri[:, 2] - tri[:, 0]
    c = np.cross(a, b).astype(F)
    return np.sqrt((c * c).sum(1, dtype=F)) * F(0.5) != 0


def load_gltf(path) -> np.ndarray:
    """Triangle soup ``[T, 9]`` float32 of a .gltf / .glb file in the
    reference's primitive order."""
    path = Path(path)
    doc, binary = _read_container(path)
    bufs = _buffers(doc, path, binary)
    meshes = []
    for m in doc.get("meshes", []):
        prims = []
        for p in m.get("primitives", []):
            if p.get("mode", 4) != 4:
                raise ValueError("only triangle lists are supported")
            pos = _accessor(doc, bufs, p["attributes"]["POSITION"], 3).astype(F)
            idx = _accessor(doc, bufs, p["indices"], 1).astype(np.int64)
            prims.append((pos, idx))
        meshes.append(prims)
    nodes = doc.get("nodes", [])
    has_parent = [False] * len(nodes)
    for n in nodes:
        for c in n.get("children", []):
            has_parent[c] = True
    out = []

    def visit(i: int, parent: np.ndarray) -> None:
        g = _mul(parent, _local(nodes[i]))
        if "mesh" in nodes[i]:
            for pos, idx in meshes[nodes[i]["mesh"]]:
                tri = _transform(g, pos)[idx[: idx.shape[0] // 3 * 3]].reshape(-1, 3, 3)
                out.append(tri[_nonzero_area(tri)].reshape(-1, 9))
        for c in nodes[i].get("children", []):
            visit(c, g)

    for i in range(len(nodes)):
        if not has_parent[i]:
            visit(i, np.eye(4, dtype=F))
    return np.concatenate(out) if out else np.zeros((0, 9), F)


def write_gltf(path, vertices: np.ndarray, faces: np.ndarray, name: str = "mesh") -> Path:
    """Writes one mesh (``vertices`` [V, 3], ``faces`` [F, 3]) as .gltf
    (embedded base64 buffer) or .glb, by the file suffix."""
    path = Path(path)
    v = np.ascontiguousarray(vertices, F).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
    # per-vertex normals (area-weighted face normals) and zero texture coordinates
    tri = v[f]
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]).astype(F)
    nrm = np.zeros_like(v)
    for k in range(3):
        np.add.at(nrm, f[:, k], fn)
    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(ln > 0, nrm / np.where(ln > 0, ln, 1), np.array([0, 1, 0], F)).astype(F)
    uv = np.zeros((v.shape[0], 2), F)
    blobs = [v.tobytes(), nrm.tobytes(), uv.tobytes(), f.tobytes()]
    offs = np.cumsum([0] + [len(b) for b in blobs]).tolist()
    data = b"".join(blobs)
    views = [{"buffer": 0, "byteOffset": offs[i], "byteLength": len(blobs[i])} for i in range(4)]
    views[3]["target"] = 34963
    for i in range(3):
        views[i]["target"] = 34962
    doc = {
        "asset": {"version": "2.0", "generator": "bvhraytracer_gb300"},
        "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0, "name": name}],
        "meshes": [{"name": name, "primitives": [{
            "attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3,
            "material": 0, "mode": 4}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [1.0, 1.0, 1.0, 1.0]}}],
        "accessors": [
            {"bufferView": 0, "componentType": 5126, "count": int(v.shape[0]), "type": "VEC3",
             "min": v.min(0).tolist() if v.size else [0, 0, 0],
             "max": v.max(0).tolist() if v.size else [0, 0, 0]},
            {"bufferView": 1, "componentType": 5126, "count": int(v.shape[0]), "type": "VEC3"},
            {"bufferView": 2, "componentType": 5126, "count": int(v.shape[0]), "type": "VEC2"},
            {"bufferView": 3, "componentType": 5125, "count": int(f.size), "type": "SCALAR"}],
        "bufferViews": views,
        "buffers": [{"byteLength": len(data)}],
    }
    if path.suffix.lower() == ".glb":
        js = json.dumps(doc).encode("utf-8")
        js += b" " * (-len(js) % 4)
        bin_ = data + b"\0" * (-len(data) % 4)
        total = 12 + 8 + len(js) + 8 + len(bin_)
        path.write_bytes(struct.pack("<III", _GLB_MAGIC, 2, total)
                         + struct.pack("<II", len(js), _CHUNK_JSON) + js
                         + struct.pack("<II", len(bin_), _CHUNK_BIN) + bin_)
    else:
        doc["buffers"][0]["uri"] = ("data:application/octet-stream;base64,"
                                    + base64.b64encode(data).decode("ascii"))
        path.write_text(json.dumps(doc))
    return path
