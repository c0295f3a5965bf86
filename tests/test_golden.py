"""The oracle against the golden fixtures of tests/golden/, which the
reference's own code produced (tests/golden/make_golden.py). Needs no
reference sources, so it pins the oracle on every machine.

The oracle traverses the reference's tree from the fixture (imported through
the host library, bvhgpu_bvh_import_compact) and must return the reference's
hit triangle, t, hit point, occlusion, per-ray counters, per-depth visits,
fullness histograms and ray-stream step data bit for bit.
"""
from pathlib import Path

import numpy as np
import pytest

import bvhraytracer_gb300 as pkg
from oracle import oracle as O

GOLDEN = sorted((Path(__file__).resolve().parent / "golden").glob("reference_*.npz"))
TREE = ("lo3", "hi3", "child_begin", "child_count", "prim_begin", "prim_count", "order48",
        "prim_ids")


def load(path):
    z = dict(np.load(path))
    tree = {k: z[k] for k in TREE}
    tree["prim_tri9"] = z["tris"][z["prim_ids"]]
    return z, tree


def test_fixtures_present():
    assert len(GOLDEN) >= 3


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_oracle_equals_reference_fixture(path):
    z, tree = load(path)
    n, l = int(z["N"]), int(z["L"])
    b = pkg.Bvh.from_compact(tree, n, l)
    ex = b.export_compact()  # the imported tree round-trips unchanged
    for k in TREE:
        if k != "order48":
            assert np.array_equal(ex[k], tree[k]), k
    cc = tree["child_count"]
    for i in np.nonzero(cc)[0]:
        assert np.array_equal(ex["order48"].reshape(-1, 3, 16)[i, :, :cc[i]],
                              tree["order48"].reshape(-1, 3, 16)[i, :, :cc[i]]), i
    cv = O.CompactView(ex)
    for batch, shadow in (("primary", False), ("shadow", True), ("ao", True)):
        rays = z[batch + "_rays"]
        o = O.trace_instrumented(cv, rays, shadow=shadow)
        assert np.array_equal(o["counters"][:, :6], z[batch + "_counters"]), batch
        assert np.array_equal(o["depth_hist"], z[batch + "_depth_hist"]), batch
        assert np.array_equal(o["fullness"], z[batch + "_fullness"]), batch
        if shadow:
            assert np.array_equal(o["occluded"], z[batch + "_occluded"]), batch
            continue
        prim = o["hits"].view(np.int32)[:, 0]
        assert np.array_equal(prim, z[batch + "_prim"])
        hit = prim >= 0
        assert np.array_equal(o["hits"][hit, 1].view(np.uint32),
                              z[batch + "_t"][hit].view(np.uint32))
        pos = O.hit_points(rays[hit], z["tris"][prim[hit]])
        assert np.array_equal(pos.view(np.uint32), z[batch + "_pos"][hit].view(np.uint32))
    w = O.trace_instrumented_steps(cv, z["wide_rays"], False, 256, 512)
    assert np.array_equal(w["step_count"], z["wide_step_count"])
    assert np.array_equal(w["steps"], z["wide_steps"])
    assert np.array_equal(w["counters"][:, :6], z["wide_counters"])
    whit = w["hits"].view(np.int32)[:, 0] >= 0
    assert np.array_equal(whit, ~np.isnan(z["wide_pos"][:, 0]))
    assert np.array_equal(w["hits"][whit, 1].view(np.uint32),
                          z["wide_t"][whit].view(np.uint32))
