"""glTF input / output: round trips of the synthetic scenes through .gltf and
.glb, the loader's traversal order and transforms on a hand-built node
hierarchy, index component types, and zero-area triangles dropped like
GameObject::iterateGo."""
import base64
import json

import numpy as np

from bvhraytracer_gb300 import gltf as G
from bvhraytracer_gb300 import scenes as S


def test_terrain_round_trip(tmp_path):
    v, f = S.terrain_mesh(16, seed=2)
    for name in ("t.gltf", "t.glb"):
        out = G.load_gltf(G.write_gltf(tmp_path / name, v, f))
        assert np.array_equal(out, v[f].reshape(-1, 9).astype(np.float32))


def test_clutter_soup_round_trip_drops_zero_area(tmp_path):
    tris = S.clutter(20, seed=5)
    v = tris.reshape(-1, 3)
    f = np.arange(v.shape[0]).reshape(-1, 3)
    # two degenerate triangles (repeated vertex) are skipped by the loader
    f2 = np.concatenate([f[:3], [[0, 0, 1]], f[3:], [[5, 5, 5]]])
    out = G.load_gltf(G.write_gltf(tmp_path / "c.glb", v, f2))
    assert np.array_equal(out, tris)


def _doc(nodes, positions, index_dtype=np.uint32, ctype=5125):
    pos = np.asarray(positions, np.float32)
    idx = np.arange(pos.shape[0], dtype=index_dtype)
    data = pos.tobytes() + idx.tobytes()
    return {
        "asset": {"version": "2.0"}, "nodes": nodes,
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "indices": 1,
                                    "material": 0}]}],
        "materials": [{}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": pos.shape[0],
                       "type": "VEC3"},
                      {"bufferView": 1, "componentType": ctype, "count": pos.shape[0],
                       "type": "SCALAR"}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": pos.nbytes},
                        {"buffer": 0, "byteOffset": pos.nbytes, "byteLength": idx.nbytes}],
        "buffers": [{"byteLength": len(data), "uri": "data:application/octet-stream;base64,"
                     + base64.b64encode(data).decode()}],
    }


def test_hierarchy_order_and_transforms(tmp_path):
    tri = [[0, 0, 0], [1, 0, 0], [0, 1, 0]]
    # node 0: parent translated by (10, 0, 0) with child node 2; node 1: a
    # second root scaled by 2; node 2: child rotated 90 degrees about z.
    s2 = np.sqrt(np.float32(0.5))
    nodes = [{"mesh": 0, "translation": [10, 0, 0], "children": [2]},
             {"mesh": 0, "scale": [2, 2, 2]},
             {"mesh": 0, "rotation": [0, 0, float(s2), float(s2)]}]
    for dt, ct in ((np.uint32, 5125), (np.uint16, 5123), (np.uint8, 5121)):
        p = tmp_path / f"h{ct}.gltf"
        p.write_text(json.dumps(_doc(nodes, tri, dt, ct)))
        out = G.load_gltf(p).reshape(-1, 3, 3)
        assert out.shape == (3, 3, 3)
        # order: root node 0, its child node 2, then root node 1
        np.testing.assert_allclose(out[0], [[10, 0, 0], [11, 0, 0], [10, 1, 0]], atol=1e-6)
        np.testing.assert_allclose(out[1], [[10, 0, 0], [10, 1, 0], [9, 0, 0]], atol=1e-6)
        np.testing.assert_allclose(out[2], [[0, 0, 0], [2, 0, 0], [0, 2, 0]], atol=1e-6)
