"""Many scenes in one persistent launch (bvhgpu_trace_jobs): per-ray results
equal the per-scene kernels' bit for bit, across scenes of different N, L,
node format and ray kind; the launch records into a CUDA graph."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bvhraytracer_gb300 as pkg  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _scenes():
    out = []
    specs = [("terrain", 20, 4, 4, "fp32"), ("clutter", 30, 8, 8, "fp32"),
             ("terrain", 40, 16, 4, "q8"), ("clutter", 80, 4, 8, "q8"),
             ("clutter", 50, 16, 16, "fp32"), ("terrain", 12, 12, 12, "fp32"),
             # widths off the gang multiples: padded node and leaf records
             ("clutter", 25, 3, 2, "fp32"), ("terrain", 16, 5, 7, "q8")]
    for i, (kind, size, n, l, fmt) in enumerate(specs):
        if kind == "terrain":
            tris = S.terrain(size, seed=i)
            c = np.array([0.5, 0.0, 0.5])
            rays = S.camera_rays(c + [0.0, 0.8, 0.8], c, 40 + 7 * i, 30 + 3 * i)
        else:
            tris = S.clutter(size, seed=i)
            rays = S.clutter_camera(size, 48 + 5 * i, 40, seed=i)
        bvh = pkg.Bvh(tris, n, l)
        out.append((tris, bvh, pkg.Scene(bvh, node_format=fmt), rays))
    return out


def _jobs(items, profile):
    jobs, refs = [], []
    for tris, bvh, scene, rays in items:
        d = torch.from_numpy(rays).cuda()
        ref_h = scene.trace(d, profile=profile)["hits"]
        prims = pkg.hit_prims(ref_h.cpu().numpy())
        m, p, n = S.surface(tris, rays, prims)
        ao = torch.from_numpy(S.ao_rays(p, n, 3, 0.1 * S.scene_diagonal(tris), seed=2)).cuda()
        ref_a = scene.trace(ao, kind="any", profile=profile)["occluded"]
        jobs.append((scene, d, "closest", torch.empty_like(ref_h)))
        jobs.append((scene, ao, "any", torch.empty_like(ref_a)))
        refs += [ref_h, ref_a]
    return jobs, refs


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
@pytest.mark.parametrize("policy", [0, 2])
@pytest.mark.parametrize("one_launch", [False, True], ids=["per_group", "one_launch"])
def test_jobs_match_per_scene_kernels(profile, policy, one_launch):
    items = _scenes()
    jobs, refs = _jobs(items, profile)
    for _ in range(2):
        for j in jobs:
            j[3].fill_(7)
        pkg.trace_jobs(jobs, profile=profile, policy=policy, one_launch=one_launch)
        torch.cuda.synchronize()
        for (scene, rays, kind, out), ref in zip(jobs, refs):
            if kind == "closest":
                assert torch.equal(out.view(torch.int32), ref.view(torch.int32))
            else:
                assert torch.equal(out, ref)
    for it in items:
        it[2].status()


def test_jobs_against_oracle():
    tris, bvh, scene, rays = _scenes()[1]
    jobs, _ = _jobs([(tris, bvh, scene, rays)], "instrumented")
    pkg.trace_jobs(jobs)
    torch.cuda.synchronize()
    ref = O.trace_instrumented(O.CompactView(bvh.export_compact()), rays, shadow=False)
    assert np.array_equal(jobs[0][3].cpu().numpy().view(np.uint32), ref["hits"].view(np.uint32))


@pytest.mark.parametrize("one_launch", [False, True], ids=["per_group", "one_launch"])
def test_jobs_in_a_cuda_graph(one_launch):
    items = _scenes()
    jobs, refs = _jobs(items, "instrumented")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        pkg.trace_jobs(jobs, stream=s, one_launch=one_launch)  # first call outside the capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        pkg.trace_jobs(jobs, one_launch=one_launch)
    for _ in range(3):
        for j in jobs:
            j[3].fill_(5)
        g.replay()
        torch.cuda.synchronize()
        for (scene, rays, kind, out), ref in zip(jobs, refs):
            if kind == "closest":
                assert torch.equal(out.view(torch.int32), ref.view(torch.int32))
            else:
                assert torch.equal(out, ref)


def test_jobs_limits():
    items = _scenes()[:1]
    jobs, _ = _jobs(items, "instrumented")
    with pytest.raises(pkg.BvhgpuError):
        pkg.trace_jobs(jobs * 100)  # 200 jobs > 192
    pkg.trace_jobs([])


@pytest.mark.parametrize("graph", [False, True])
def test_reordered_jobs(graph):
    """Jobs whose rays are grouped by direction first (per-job segmented
    counting sort, results back in input order) equal the per-scene traces,
    eagerly and recorded in a CUDA graph (the scratch is stream-ordered)."""
    items = _scenes()
    jobs, refs = _jobs(items, "instrumented")
    jobs = [j + ((8 if j[2] == "any" or i % 4 == 0 else 0),) for i, j in enumerate(jobs)]

    def check():
        for (scene, rays, kind, out, _), ref in zip(jobs, refs):
            if kind == "closest":
                assert torch.equal(out.view(torch.int32), ref.view(torch.int32))
            else:
                assert torch.equal(out, ref)

    if not graph:
        for one_launch in (False, True):
            for j in jobs:
                j[3].fill_(7)
            pkg.trace_jobs(jobs, policy=2, refill=24, one_launch=one_launch)
            torch.cuda.synchronize()
            check()
        with pytest.raises(pkg.BvhgpuError):
            pkg.trace_jobs([jobs[1], jobs[3][:4] + (10,)])  # reordered jobs must share K
        return
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        pkg.trace_jobs(jobs, stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        pkg.trace_jobs(jobs)
    for _ in range(2):
        for j in jobs:
            j[3].fill_(5)
        g.replay()
        torch.cuda.synchronize()
        check()


@pytest.mark.parametrize("profile", ["instrumented", "fast"])
def test_jobs_any_order(profile):
    """Any-hit jobs with child-index push order (per job) equal the
    per-scene traces, next to jobs in the reference's order."""
    items = _scenes()
    jobs, refs = _jobs(items, profile)
    jobs = [j + ((8 if i % 3 == 1 else 0), i % 2) for i, j in enumerate(jobs)]
    for j in jobs:
        j[3].fill_(3)
    pkg.trace_jobs(jobs, profile=profile, policy=2, refill=24)
    torch.cuda.synchronize()
    for (scene, rays, kind, out, _, _), ref in zip(jobs, refs):
        if kind == "closest":
            assert torch.equal(out.view(torch.int32), ref.view(torch.int32))
        else:
            assert torch.equal(out, ref)


@pytest.mark.parametrize("kind", ["closest", "any"])
def test_jobs_of_one_kind(kind):
    """A job list of one ray kind (one launch, kernel compiled for that
    kind) and of one kind and node width (one group) equal the per-scene
    traces."""
    items = _scenes()
    jobs, refs = _jobs(items, "instrumented")
    sel = [(j, r) for j, r in zip(jobs, refs) if j[2] == kind]
    for subset in (sel, [x for x in sel if x[0][0].node_format == "fp32"][:2]):
        for one_launch in (False, True):
            for j, _ in subset:
                j[3].fill_(9)
            pkg.trace_jobs([j for j, _ in subset], policy=2, refill=16, one_launch=one_launch)
            torch.cuda.synchronize()
            for (scene, rays, k, out), ref in subset:
                assert torch.equal(out.view(torch.uint8), ref.view(torch.uint8))
