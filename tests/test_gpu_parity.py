"""GPU parity: the sm_103a kernels against the CPU oracle, bit for bit
(hit primitive, t, barycentrics, per-ray counters, per-depth histograms),
for both traversal schemes, both profiles and every N, L in {4,8,12,16}."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests import _scenes as TS  # noqa: E402

pytestmark = pytest.mark.gpu

LIGHT = [2.0, 3.0, 2.0]
# (scheme, extra trace options): every traversal scheme and persistent policy
SCHEMES = [("per_ray", {}), ("stream", {}), ("persistent", {"policy": 0}),
           ("persistent", {"policy": 1, "refill": 1}), ("persistent", {"policy": 2, "refill": 16}),
           ("persistent", {"policy": 3, "refill": 24}), ("persistent", {"policy": 4, "refill": 24})]
SCHEME_IDS = ["per_ray", "stream", "persistent_ww", "persistent_ifif_r1", "persistent_spec",
              "persistent_spec2", "persistent_coop"]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def check_closest(got, ref, counters=True):
    g = got["hits"].cpu().numpy()
    assert np.array_equal(bits(g), bits(ref["hits"])), _first_diff(g, ref["hits"])
    if counters:
        gc = got["counters"].cpu().numpy().astype(np.uint32)[:, :7]
        assert np.array_equal(gc, ref["counters"][:, :7])
        assert np.array_equal(got["depth_hist"].cpu().numpy().astype(np.uint64), ref["depth_hist"])
        if ref.get("fullness") is not None:
            assert np.array_equal(got["fullness"].cpu().numpy().astype(np.uint64), ref["fullness"])


def check_any(got, ref, counters=True):
    assert np.array_equal(got["occluded"].cpu().numpy(), ref["occluded"])
    if counters:
        gc = got["counters"].cpu().numpy().astype(np.uint32)[:, :7]
        assert np.array_equal(gc, ref["counters"][:, :7])
        assert np.array_equal(got["depth_hist"].cpu().numpy().astype(np.uint64), ref["depth_hist"])
        if ref.get("fullness") is not None:
            assert np.array_equal(got["fullness"].cpu().numpy().astype(np.uint64), ref["fullness"])


def _first_diff(g, r):
    d = np.nonzero(np.any(bits(g) != bits(r), axis=1))[0]
    if d.size == 0:
        return "equal"
    i = d[0]
    return f"{d.size} rays differ; first {i}: gpu {g[i].view(np.int32)[0]} {g[i][1:]} " \
           f"oracle {r[i].view(np.int32)[0]} {r[i][1:]}"


@pytest.fixture(scope="module")
def terrain():
    tris, b, cv = TS.bvh("terrain", 4, 4)
    rays = TS.terrain_case()[1]
    return tris, b, cv, rays, pkg.Scene(b)


@pytest.mark.parametrize("scheme,kw", SCHEMES, ids=SCHEME_IDS)
def test_terrain_instrumented_primary_and_shadow(terrain, scheme, kw):
    tris, b, cv, rays, scene = terrain
    ref = O.trace_instrumented(cv, rays, shadow=False)
    got = scene.trace(dev(rays), scheme=scheme, counters=True, depth_hist=True, **kw)
    check_closest(got, ref)
    prims = pkg.hit_prims(ref["hits"])
    sh, _ = TS.secondary(tris, rays, prims, LIGHT)
    refs = O.trace_instrumented(cv, sh, shadow=True)
    gots = scene.trace(dev(sh), kind="any", scheme=scheme, counters=True, depth_hist=True, **kw)
    check_any(gots, refs)
    # the fast (counter-free) kernels give the same hits
    check_closest(scene.trace(dev(rays), scheme=scheme, **kw), ref, counters=False)
    check_any(scene.trace(dev(sh), kind="any", scheme=scheme, **kw), refs, counters=False)
    scene.status()


@pytest.mark.parametrize("scheme,kw", SCHEMES, ids=SCHEME_IDS)
def test_terrain_fast_profile(terrain, scheme, kw):
    tris, b, cv, rays, scene = terrain
    fv = O.FastView(b.export_fast())
    ref = O.trace_fast(fv, cv, rays, any_hit=False)
    got = scene.trace(dev(rays), scheme=scheme, profile="fast", counters=True, depth_hist=True,
                      **kw)
    check_closest(got, ref)
    prims = pkg.hit_prims(ref["hits"])
    sh, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=2)
    for sec in (sh, ao):
        r = O.trace_fast(fv, cv, sec, any_hit=True)
        g = scene.trace(dev(sec), kind="any", scheme=scheme, profile="fast", counters=True,
                        depth_hist=True, **kw)
        check_any(g, r)


@pytest.mark.parametrize("n", [4, 8, 12, 16])
@pytest.mark.parametrize("l", [4, 8, 12, 16])
def test_sweep_all_widths(n, l):
    tris, b, cv = TS.bvh("clutter120", n, l)
    rays = TS.clutter_rays(tris, res=(64, 48))
    scene = pkg.Scene(b)
    fv = O.FastView(b.export_fast())
    for profile in ("instrumented", "fast"):
        if profile == "instrumented":
            ref = O.trace_instrumented(cv, rays, shadow=False)
        else:
            ref = O.trace_fast(fv, cv, rays, any_hit=False)
        prims = pkg.hit_prims(ref["hits"])
        _, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=2)
        if profile == "instrumented":
            refa = O.trace_instrumented(cv, ao, shadow=True)
        else:
            refa = O.trace_fast(fv, cv, ao, any_hit=True)
        for scheme, kw in SCHEMES:
            got = scene.trace(dev(rays), scheme=scheme, profile=profile, counters=True,
                              depth_hist=True, **kw)
            check_closest(got, ref)
            g = scene.trace(dev(ao), kind="any", scheme=scheme, profile=profile, counters=True,
                            depth_hist=True, **kw)
            check_any(g, refa)
            check_closest(scene.trace(dev(rays), scheme=scheme, profile=profile, **kw), ref, False)
            check_any(scene.trace(dev(ao), kind="any", scheme=scheme, profile=profile, **kw),
                      refa, False)


@pytest.mark.parametrize("n,l", [(2, 1), (3, 2), (5, 3), (7, 5), (9, 7), (13, 11), (2, 16),
                                 (16, 1)])
def test_odd_widths(n, l):
    """Branching factors and leaf sizes off the gang multiples (the reference's
    render-time sweeps run N = 2..16, LatexPlots/MatLibPlot/PerformancePlots.py:21-24):
    node and leaf records are padded to the gang of 4 like
    fastNodeManager.h:1556,1602, the padding lanes never hit. Every scheme,
    both profiles, closest and any hit, counters included; Q8 nodes keep the
    hits."""
    tris, b, cv = TS.bvh("clutter120", n, l)
    rays = TS.clutter_rays(tris, res=(64, 48))
    scene = pkg.Scene(b)
    fv = O.FastView(b.export_fast())
    for profile in ("instrumented", "fast"):
        if profile == "instrumented":
            ref = O.trace_instrumented(cv, rays, shadow=False)
        else:
            ref = O.trace_fast(fv, cv, rays, any_hit=False)
        prims = pkg.hit_prims(ref["hits"])
        _, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=2)
        if profile == "instrumented":
            refa = O.trace_instrumented(cv, ao, shadow=True)
        else:
            refa = O.trace_fast(fv, cv, ao, any_hit=True)
        for scheme, kw in SCHEMES:
            got = scene.trace(dev(rays), scheme=scheme, profile=profile, counters=True,
                              depth_hist=True, **kw)
            check_closest(got, ref)
            g = scene.trace(dev(ao), kind="any", scheme=scheme, profile=profile, counters=True,
                            depth_hist=True, **kw)
            check_any(g, refa)
        s8 = pkg.Scene(b, node_format="q8")
        for scheme, kw in (("per_ray", {}), ("persistent", {"policy": 2, "refill": 16})):
            got = s8.trace(dev(rays), scheme=scheme, profile=profile, **kw)
            check_closest(got, ref, False)
            check_any(s8.trace(dev(ao), kind="any", scheme=scheme, profile=profile, **kw), refa,
                      False)
        s8.status()
    scene.status()


@pytest.mark.parametrize("gang,leaf_memory", [(8, 0), (4, 16), (8, 16)])
def test_gang_and_leaf_memory(gang, leaf_memory):
    tris, b, cv = TS.bvh("clutter120", 8, 4)
    rays = TS.clutter_rays(tris, res=(64, 48))
    scene = pkg.Scene(b, gang=gang, leaf_memory=leaf_memory)
    fv = O.FastView(b.export_fast(gang=gang, leaf_memory=leaf_memory))
    ref = O.trace_fast(fv, cv, rays, any_hit=False)
    for scheme, kw in SCHEMES:
        check_closest(scene.trace(dev(rays), scheme=scheme, profile="fast", counters=True,
                                  depth_hist=True, **kw), ref)
    ref = O.trace_instrumented(cv, rays, shadow=False)
    check_closest(scene.trace(dev(rays), counters=True, depth_hist=True), ref)


@pytest.mark.parametrize("top_levels", [1, 2, 3])
def test_top_levels_layout(top_levels):
    tris, b, cv = TS.bvh("clutter120", 4, 4)
    rays = TS.clutter_rays(tris, res=(64, 48))
    ref = O.trace_instrumented(cv, rays, shadow=False)
    scene = pkg.Scene(b, top_levels=top_levels)
    for scheme, kw in SCHEMES:
        check_closest(scene.trace(dev(rays), scheme=scheme, counters=True, depth_hist=True, **kw),
                      ref)


def test_edge_cases():
    # single triangle: the root is a leaf
    t1 = np.array([[0, 0, 5, 1, 0, 5, 0, 1, 5]], np.float32)
    b = pkg.Bvh(t1, 4, 4)
    cv = O.CompactView(b.export_compact())
    scene = pkg.Scene(b)
    rays = np.array([[0.25, 0.25, 0, 222222, 0, 0, 1, 0],     # hit, zero x/y direction
                     [0.75, 0.75, 0, 222222, 0, 0, 1, 0],     # miss
                     [np.nan, 0, 0, 222222, 0, 0, 1, 0],      # inactive
                     [0.25, 0.25, 0, 4.0, 0, 0, 1, 0],        # tmax too short
                     [0.25, 0.25, 10, 222222, 0, 0, -3, 0]],  # from behind, long direction
                    np.float32)
    for scheme, kw in SCHEMES:
        got = scene.trace(dev(rays), scheme=scheme, counters=True, depth_hist=True, **kw)
        ref = O.trace_instrumented(cv, rays, shadow=False)
        check_closest(got, ref)
        assert pkg.hit_prims(got["hits"].cpu().numpy()).tolist() == [0, -1, -1, -1, 0]
        occ = scene.trace(dev(rays), kind="any", scheme=scheme, **kw)["occluded"].cpu().numpy()
        assert occ.tolist() == [1, 0, 0, 0, 1]
    # empty batch
    e = scene.trace(dev(np.zeros((0, 8), np.float32)))
    assert e["hits"].shape == (0, 4)


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
def test_non_finite_and_extreme_rays(profile):
    """Rays the renderer never makes but a caller may pass: infinite and
    zero tMax, NaN or infinite direction components, a zero direction,
    signed zeros, subnormal and huge components, origins far outside the
    scene. Every scheme returns the oracle's results (the reference's
    comparison forms decide what a NaN does): bit for bit, except that a NaN
    result matches any NaN (the GPU's canonical NaN is 0x7fffffff, an x86
    host's default NaN 0xffc00000)."""

    def nan_bits(hits):
        # (prim, t, u, v): prim compared as is, t / u / v with one NaN pattern
        u = np.ascontiguousarray(hits, np.float32).view(np.uint32).copy()
        f = np.ascontiguousarray(hits, np.float32)
        u[:, 1:][np.isnan(f[:, 1:])] = 0x7FC00000
        return u
    tris, b, cv = TS.bvh("clutter120", 8, 4)
    fv = O.FastView(b.export_fast()) if profile == "fast" else None
    base = TS.clutter_rays(tris)[:64].copy()
    rows = []
    inf, nan = np.float32(np.inf), np.float32(np.nan)
    for k, r in enumerate(base):
        r = r.copy()
        v = k % 16
        if v == 0: r[3] = inf
        elif v == 1: r[3] = 0.0
        elif v == 2: r[5] = nan
        elif v == 3: r[4:7] = 0.0
        elif v == 4: r[4] = -0.0; r[5] = 0.0
        elif v == 5: r[6] = inf
        elif v == 6: r[4:7] *= np.float32(1e-40)
        elif v == 7: r[4:7] *= np.float32(1e30)
        elif v == 8: r[0:3] = np.float32(1e30)
        elif v == 9: r[0:3] = -r[0:3] * 100
        elif v == 10: r[3] = nan
        elif v == 11: r[1] = inf
        elif v == 12: r[3] = -1.0
        elif v == 13: r[4] = np.float32(1e-45)
        rows.append(r)
    rays = np.stack(rows).astype(np.float32)
    scene = pkg.Scene(b)
    for kind in ("closest", "any"):
        if profile == "instrumented":
            ref = O.trace_instrumented(cv, rays, shadow=kind == "any", counters=False)
        else:
            ref = O.trace_fast(fv, cv, rays, any_hit=kind == "any", counters=False)
        for scheme, kw in SCHEMES:
            got = scene.trace(dev(rays), kind=kind, scheme=scheme, profile=profile, **kw)
            if kind == "closest":
                assert np.array_equal(nan_bits(got["hits"].cpu().numpy()),
                                      nan_bits(ref["hits"])), scheme
            else:
                assert np.array_equal(got["occluded"].cpu().numpy(), ref["occluded"]), scheme
        extra = [{"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 8}]
        if kind == "any":
            extra.append({"scheme": "persistent", "policy": 2, "refill": 24, "any_order": True})
        for o in extra:
            got = scene.trace(dev(rays), kind=kind, profile=profile, **o)
            if kind == "closest":
                assert np.array_equal(nan_bits(got["hits"].cpu().numpy()),
                                      nan_bits(ref["hits"])), o
            else:
                assert np.array_equal(got["occluded"].cpu().numpy(), ref["occluded"]), o
    if profile == "instrumented":
        got = scene.trace(dev(rays), counters=True, depth_hist=True)
        ref = O.trace_instrumented(cv, rays, shadow=False)
        assert np.array_equal(nan_bits(got["hits"].cpu().numpy()), nan_bits(ref["hits"]))
        assert np.array_equal(got["counters"].cpu().numpy().astype(np.uint32)[:, :7],
                              ref["counters"][:, :7])
        assert np.array_equal(got["depth_hist"].cpu().numpy().astype(np.uint64),
                              ref["depth_hist"])
    scene.status()


@pytest.mark.parametrize("kind,n,l", [("terrain", 4, 4), ("clutter120", 8, 4),
                                      ("clutter120", 16, 16)])
def test_stream_step_log(kind, n, l):
    """bvhgpu_trace_steps: per packet and step the node work, unique nodes,
    leaf work, unique leaves and terminations of intersectWideAlternative
    (and of intersectWide's schedule) equal the oracle's, for primary and
    shadow rays (inactive rays, a ragged last packet, a step log shorter than
    the traversal)."""
    tris, b, cv = TS.bvh(kind, n, l)
    rays = (TS.terrain_case()[1] if kind == "terrain" else TS.clutter_rays(tris))[:-77]
    scene = pkg.Scene(b)
    prims = pkg.hit_prims(scene.trace(dev(rays))["hits"].cpu().numpy())
    sh, _ = TS.secondary(tris, rays, prims, LIGHT)
    cap = 400
    for (shadow, r), alt in [(x, y) for x in ((False, rays), (True, sh)) for y in (True, False)]:
        ref = O.trace_instrumented_steps(cv, r, shadow, 256, cap, wide_alternative=alt)
        assert int(ref["step_count"].max()) < cap
        got = scene.trace(dev(r), kind="any" if shadow else "closest", scheme="stream",
                          counters=True, depth_hist=True, steps=cap, wide_alternative=alt)
        assert np.array_equal(got["step_count"].cpu().numpy().astype(np.uint32),
                              ref["step_count"])
        assert np.array_equal(got["step_stats"].cpu().numpy().astype(np.uint32), ref["steps"])
        assert np.array_equal(got["counters"].cpu().numpy().astype(np.uint32)[:, :7],
                              ref["counters"][:, :7])
        if shadow:
            assert np.array_equal(got["occluded"].cpu().numpy(), ref["occluded"])
        else:
            assert np.array_equal(bits(got["hits"].cpu().numpy()), bits(ref["hits"]))
        short = scene.trace(dev(r), kind="any" if shadow else "closest", scheme="stream",
                            counters=True, steps=3, wide_alternative=alt)
        assert np.array_equal(short["step_count"].cpu().numpy().astype(np.uint32),
                              ref["step_count"])
        assert np.array_equal(short["step_stats"].cpu().numpy().astype(np.uint32),
                              ref["steps"][:, :3])
    with pytest.raises(pkg.BvhgpuError):
        scene.trace(dev(rays), scheme="per_ray", counters=True, steps=8)
    with pytest.raises(pkg.BvhgpuError):
        scene.trace(dev(rays), scheme="stream", steps=8)
    scene.status()


@pytest.mark.parametrize("n", [1, 31, 127, 129, 255, 257, 1000])
def test_ragged_ray_counts(n, terrain):
    tris, b, cv, rays, scene = terrain
    r = rays[40000:40000 + n]
    ref = O.trace_instrumented(cv, r, shadow=False)
    for scheme, kw in SCHEMES:
        check_closest(scene.trace(dev(r), scheme=scheme, counters=True, depth_hist=True, **kw),
                      ref)


def test_host_entry_point_matches_device(terrain):
    tris, b, cv, rays, scene = terrain
    ref = O.trace_instrumented(cv, rays, shadow=False)
    out = scene.trace_host(rays)
    assert np.array_equal(bits(out), bits(ref["hits"]))
    prims = pkg.hit_prims(ref["hits"])
    sh, _ = TS.secondary(tris, rays, prims, LIGHT)
    occ = scene.trace_host(sh, kind="any", scheme="stream")
    assert np.array_equal(occ, O.trace_instrumented(cv, sh, shadow=True)["occluded"])


def test_host_batches_in_one_pipeline(terrain):
    """bvhgpu_trace_host_batches: primary, shadow and AO batches with their
    own options in one pipelined call (ragged sizes, an empty batch, more
    than one chunk for the largest) equal the oracle."""
    tris, b, cv, rays, scene = terrain
    ref = O.trace_instrumented(cv, rays, shadow=False)
    prims = pkg.hit_prims(ref["hits"])
    sh, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=8)
    big = np.concatenate([ao] * 24)  # > 256 Ki rays: several chunks
    outs = scene.trace_host_batches([
        (rays[:-3], "closest", None, {"scheme": "per_ray", "stack": "local"}),
        (sh, "any", None, {"scheme": "persistent", "policy": 2, "refill": 16}),
        (rays[:0], "closest", None, {}),
        (big, "any", None, {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10,
                            "any_order": True}),
        (ao, "any", None, {"scheme": "stream"})])
    assert np.array_equal(bits(outs[0]), bits(ref["hits"][:-3]))
    occ_sh = O.trace_instrumented(cv, sh, shadow=True)["occluded"]
    occ_ao = O.trace_instrumented(cv, ao, shadow=True)["occluded"]
    assert np.array_equal(outs[1], occ_sh)
    assert outs[2].shape == (0, 4)
    assert np.array_equal(outs[3], np.concatenate([occ_ao] * 24))
    assert np.array_equal(outs[4], occ_ao)
    with pytest.raises(pkg.BvhgpuError):
        scene.trace_host_batches([(sh, "any", None, {"reorder": 40})])


def test_wrappers_mirror_reference_names(terrain):
    tris, b, cv, rays, scene = terrain
    fm = pkg.FastNodeManager(b)
    fv = O.FastView(b.export_fast())
    ref = O.trace_fast(fv, cv, rays, any_hit=False)
    for fn in (fm.intersect, fm.intersect_wide_alternative):
        assert np.array_equal(bits(fn(dev(rays)).cpu().numpy()), bits(ref["hits"]))
    cm = pkg.CompactNodeManager(b)
    refi = O.trace_instrumented(cv, rays, shadow=False)
    for fn in (cm.intersect_immediately, cm.intersect_wide_alternative):
        check_closest(fn(dev(rays)), refi)


def test_full_size_clutter_properties():
    """1M-triangle clutter, N8L8, 1920x1080 primary rays: per-ray and stream
    kernels agree bit for bit on every ray; a random sample agrees with the
    oracle; any-hit == (closest hit within tmax) for the AO rays."""
    tris = TS.clutter_tris(4000, 1)
    b = pkg.Bvh(tris, 8, 8)
    scene = pkg.Scene(b)
    rays = S.clutter_camera(4000, 1920, 1080)
    d = dev(rays)
    a = scene.trace(d)["hits"]
    for scheme, kw in SCHEMES[1:]:
        s = scene.trace(d, scheme=scheme, **kw)["hits"]
        assert torch.equal(a.view(torch.int32), s.view(torch.int32)), scheme
    cv = O.CompactView(b.export_compact())
    idx = np.random.default_rng(0).choice(rays.shape[0], 20000, replace=False)
    ref = O.trace_instrumented(cv, rays[idx], shadow=False)
    assert np.array_equal(bits(a.cpu().numpy()[idx]), bits(ref["hits"]))
    prims = pkg.hit_prims(a.cpu().numpy())
    _, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=2)
    da = dev(ao)
    occ = scene.trace(da, kind="any")["occluded"]
    for scheme, kw in SCHEMES[1:]:
        assert torch.equal(occ, scene.trace(da, kind="any", scheme=scheme, **kw)["occluded"])
    close = scene.trace(da)["hits"]
    assert torch.equal(occ.bool(), close.view(torch.int32)[:, 0] >= 0)
    scene.status()
    # Q8 nodes with the top levels staged in shared memory: identical hits.
    q8 = pkg.Scene(b, node_format="q8", top_levels=2)
    assert torch.equal(q8.trace(d, scheme="persistent")["hits"].view(torch.int32),
                       a.view(torch.int32))
    assert torch.equal(q8.trace(da, kind="any", scheme="persistent")["occluded"], occ)
    q8.status()


def _fastrays(rays):
    """FastRay records (tMax, pos, invDirection, direction) like FastRay::FastRay."""
    fr = np.zeros((rays.shape[0], 10), np.float32)
    fr[:, 0] = rays[:, 3]
    fr[:, 1:4] = rays[:, 0:3]
    d = rays[:, 4:7]
    with np.errstate(divide="ignore"):
        inv = np.float32(1.0) / d
    inv[d == 0] = np.finfo(np.float32).max
    fr[:, 4:7] = inv
    fr[:, 7:10] = d
    return fr


@pytest.mark.parametrize("scheme", [pkg.PER_RAY, pkg.STREAM])
def test_fastray_drop_in(terrain, scheme):
    """bvhgpu_intersect_fastrays / _secondary_fastrays against the oracle's
    FastNodeManager restatement: leafIndex, triIndex, tMax and AO counts."""
    import ctypes as C
    from bvhraytracer_gb300 import _native as N
    tris, b, cv, rays, scene = terrain
    fv = O.FastView(b.export_fast())
    ref = O.trace_fast(fv, cv, rays, any_hit=False)
    fr = _fastrays(rays)
    li = np.full(rays.shape[0], 7, np.uint32)
    ti = np.zeros(rays.shape[0], np.int8)
    N.check(N.lib().bvhgpu_intersect_fastrays(scene.handle, fr.ctypes.data, rays.shape[0], scheme,
                                              li.ctypes.data, ti.ctypes.data, None))
    hit = ref["tri_index"] >= 0
    assert np.array_equal(ti, ref["tri_index"])
    assert np.array_equal(li[hit], ref["leaf_index"][hit].astype(np.uint32))
    assert np.all(li[~hit] == 7)
    assert np.array_equal(fr[:, 0].view(np.uint32), ref["hits"][:, 1].view(np.uint32))
    prims = pkg.hit_prims(ref["hits"])
    _, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=2)
    res = np.full(ao.shape[0], 3, np.uint16)
    fa = _fastrays(ao)
    N.check(N.lib().bvhgpu_intersect_secondary_fastrays(scene.handle, fa.ctypes.data, ao.shape[0],
                                                        scheme, res.ctypes.data, None))
    occ = O.trace_fast(fv, cv, ao, any_hit=True)["occluded"]
    assert np.array_equal(res, 3 + occ.astype(np.uint16))


@pytest.mark.parametrize("n,l", [(4, 4), (8, 8), (16, 16), (8, 4), (12, 8)])
def test_q8_nodes_keep_hits_identical(n, l):
    """8-bit child boxes relative to the parent box, rounded outward: the
    hit sets (and every closest-hit record) equal the FP32 nodes' and the
    oracle's; node bytes shrink."""
    tris, b, cv = TS.bvh("clutter120", n, l)
    rays = TS.clutter_rays(tris, res=(96, 64))
    s32 = pkg.Scene(b)
    s8 = pkg.Scene(b, node_format="q8", top_levels=2)
    assert s8.node_bytes < s32.node_bytes
    for profile in ("instrumented", "fast"):
        ref = s32.trace(dev(rays), profile=profile)["hits"].cpu().numpy()
        prims = pkg.hit_prims(ref)
        sh, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=2)
        ref_a = s32.trace(dev(ao), kind="any", profile=profile)["occluded"].cpu().numpy()
        for scheme, kw in (("per_ray", {}), ("persistent", {"policy": 0}),
                           ("persistent", {"policy": 1}), ("persistent", {"policy": 2})):
            got = s8.trace(dev(rays), scheme=scheme, profile=profile, **kw)["hits"].cpu().numpy()
            assert np.array_equal(bits(got), bits(ref)), (profile, scheme, _first_diff(got, ref))
            occ = s8.trace(dev(ao), kind="any", scheme=scheme, profile=profile, **kw)["occluded"]
            assert np.array_equal(occ.cpu().numpy(), ref_a), (profile, scheme)
    # counters run on Q8 too (visits may grow: boxes are conservative)
    c8 = s8.trace(dev(rays), counters=True)["counters"].cpu().numpy()
    c32 = s32.trace(dev(rays), counters=True)["counters"].cpu().numpy()
    assert c8[:, 0].sum() >= c32[:, 0].sum()
    s8.status()
    with pytest.raises(pkg.BvhgpuError):
        s8.trace(dev(rays), scheme="stream")


@pytest.mark.parametrize("n,l", [(4, 4), (8, 8), (16, 4)])
@pytest.mark.parametrize("profile", ["instrumented", "fast"])
@pytest.mark.parametrize("fmt", ["fp32", "q8"])
def test_save_distance_traversal(n, l, profile, fmt):
    """intersectSaveDistance / intersectImmediately(ray, useDistance=true):
    hits, counters and depth histograms bit-exact against the oracle; any-hit
    rays are unaffected."""
    tris, b, cv = TS.bvh("clutter120", n, l)
    fv = O.FastView(b.export_fast())
    rays = TS.clutter_rays(tris)
    scene = pkg.Scene(b, node_format=fmt)
    if profile == "instrumented":
        ref = O.trace_instrumented(cv, rays, False, use_distance=True)
    else:
        ref = O.trace_fast(fv, cv, rays, False, use_distance=True)
    got = scene.trace(dev(rays), profile=profile, save_distance=True, counters=True,
                      depth_hist=True)
    if fmt == "fp32":
        check_closest(got, ref)
    check_closest(scene.trace(dev(rays), profile=profile, save_distance=True), ref,
                  counters=False)
    prims = pkg.hit_prims(ref["hits"])
    _, ao = TS.secondary(tris, rays, prims, LIGHT)
    plain = scene.trace(dev(ao), kind="any", profile=profile)["occluded"]
    dist = scene.trace(dev(ao), kind="any", profile=profile, save_distance=True)["occluded"]
    assert torch.equal(plain, dist)
    with pytest.raises(pkg.BvhgpuError):
        scene.trace(dev(rays), scheme="persistent", save_distance=True)
    scene.status()


@pytest.mark.parametrize("scheme,kw", [("per_ray", {}), ("persistent", {"policy": 2, "refill": 16}),
                                       ("stream", {})], ids=["per_ray", "persistent", "stream"])
@pytest.mark.parametrize("k", [1, 8, 32])
def test_reorder_keeps_results_in_input_order(scheme, kw, k):
    """reorder = K traces the rays grouped into 6 K^2 direction bins; hits,
    occlusion and counters come back in input order, equal to the plain
    trace; inactive (NaN) rays and a ragged count included."""
    tris, b, cv = TS.bvh("clutter120", 8, 8)
    rays = TS.clutter_rays(tris)[:5000 - 3].copy()
    rays[::97, 0] = np.nan
    scene = pkg.Scene(b)
    d = dev(rays)
    plain = scene.trace(d, scheme=scheme, counters=True, **kw)
    got = scene.trace(d, scheme=scheme, counters=True, reorder=k, **kw)
    assert torch.equal(plain["hits"].view(torch.int32), got["hits"].view(torch.int32))
    assert torch.equal(plain["counters"], got["counters"])
    prims = pkg.hit_prims(plain["hits"].cpu().numpy())
    _, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=4)
    da = dev(ao)
    occ = scene.trace(da, kind="any", scheme=scheme, **kw)["occluded"]
    occ_r = scene.trace(da, kind="any", scheme=scheme, reorder=k, **kw)["occluded"]
    assert torch.equal(occ, occ_r)
    ref = O.trace_instrumented(cv, ao, shadow=True, counters=False)["occluded"]
    assert np.array_equal(occ_r.cpu().numpy(), ref)
    one = scene.trace(d[:1], reorder=k)["hits"]
    assert torch.equal(one.view(torch.int32), plain["hits"][:1].view(torch.int32))
    host = scene.trace_host(ao, kind="any", reorder=k)
    assert np.array_equal(host, ref)
    with pytest.raises(pkg.BvhgpuError):
        scene.trace(d, reorder=33)
    scene.status()


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
@pytest.mark.parametrize("fmt", ["fp32", "q8"])
def test_any_order_keeps_any_hit_results(profile, fmt):
    """any_order: any-hit rays without counters push hit children in
    child-index order in both profiles; occlusion equals the oracle's for
    every scheme (shadow and AO rays, inactive rays included), and traces
    with counters keep the reference's order and counts."""
    tris, b, cv = TS.bvh("clutter120", 8, 4)
    fv = O.FastView(b.export_fast()) if profile == "fast" else None
    rays = TS.clutter_rays(tris)[:3000 - 5].copy()
    scene = pkg.Scene(b, node_format=fmt)
    prims = pkg.hit_prims(scene.trace(dev(rays), profile=profile)["hits"].cpu().numpy())
    shadow, ao = TS.secondary(tris, rays, prims, LIGHT, ao_samples=4)
    for sec in (shadow, ao):
        sec = sec.copy()
        sec[::89, 0] = np.nan
        if profile == "instrumented":
            ref = O.trace_instrumented(cv, sec, shadow=True, counters=False)["occluded"]
        else:
            ref = O.trace_fast(fv, cv, sec, any_hit=True, counters=False)["occluded"]
        d = dev(sec)
        for scheme, kw in (("per_ray", {}), ("per_ray", {"stack": "local"}),
                           ("stream", {}), ("persistent", {"policy": 0, "refill": 8}),
                           ("persistent", {"policy": 2, "refill": 24, "reorder": 10}),
                           ("persistent", {"policy": 3, "refill": 24, "reorder": 10}),
                           ("persistent", {"policy": 4, "refill": 24, "reorder": 10}),
                           ("persistent", {"policy": 4, "refill": 8})):
            if fmt == "q8" and scheme == "stream":
                continue
            got = scene.trace(d, kind="any", scheme=scheme, profile=profile, any_order=True,
                              **kw)["occluded"]
            assert np.array_equal(got.cpu().numpy(), ref), (scheme, kw)
        c0 = scene.trace(d, kind="any", profile=profile, counters=True)
        c1 = scene.trace(d, kind="any", profile=profile, counters=True, any_order=True)
        assert torch.equal(c0["counters"], c1["counters"])
        assert torch.equal(c0["occluded"], c1["occluded"])
        host = scene.trace_host(sec, kind="any", profile=profile, scheme="persistent", policy=2,
                                refill=24, any_order=True)
        assert np.array_equal(host, ref)
    scene.status()


@pytest.mark.parametrize("n,l", [(4, 4), (8, 8), (12, 4), (16, 16)])
def test_device_q8_encoding_matches_host(n, l):
    """Q8 scenes encode their node records on the device; the bytes equal the
    host layout builder's, which is the format's specification."""
    tris, b, _ = TS.bvh("clutter120", n, l)
    for fmt, top in (("q8", 0), ("q8", 2), ("fp32", 0)):
        sc = pkg.Scene(b, node_format=fmt, top_levels=top)
        assert np.array_equal(sc.node_records(), b.node_records(node_format=fmt, top_levels=top))
        nm = -(-n // 4) * 4
        want = {"q8": {4: 64, 8: 80, 12: 112, 16: 144}, "fp32": {4: 128, 8: 240, 12: 368,
                                                                 16: 464}}[fmt][nm]
        assert sc.node_record_bytes == want


def test_imported_tree_traces_like_the_built_one():
    """A scene made from CompactNodeV3 arrays handed over by another builder
    (here: this builder's export) traces bit for bit like the original."""
    tris, b, cv = TS.bvh("clutter120", 8, 8)
    b2 = pkg.Bvh.from_compact(b.export_compact(), 8, 8)
    rays = dev(TS.clutter_rays(tris))
    a = pkg.Scene(b).trace(rays, counters=True)
    c = pkg.Scene(b2).trace(rays, counters=True)
    assert torch.equal(a["hits"].view(torch.int32), c["hits"].view(torch.int32))
    assert torch.equal(a["counters"], c["counters"])


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
def test_local_memory_stacks(profile):
    """The stack-placement knob: per-thread stacks in local memory give the
    same results as shared-memory stacks (closest and any hit)."""
    tris, b, cv = TS.bvh("clutter120", 8, 8)
    rays = dev(TS.clutter_rays(tris))
    scene = pkg.Scene(b)
    a = scene.trace(rays, profile=profile)["hits"]
    c = scene.trace(rays, profile=profile, stack="local")["hits"]
    assert torch.equal(a.view(torch.int32), c.view(torch.int32))
    prims = pkg.hit_prims(a.cpu().numpy())
    _, ao = TS.secondary(tris, TS.clutter_rays(tris), prims, LIGHT)
    d = dev(ao)
    assert torch.equal(scene.trace(d, kind="any", profile=profile)["occluded"],
                       scene.trace(d, kind="any", profile=profile, stack="local")["occluded"])
    with pytest.raises(pkg.BvhgpuError):
        scene.trace(rays, scheme="persistent", stack="local")
