"""Benchmark: Mrays/s of BVH traversal on one GB300 (and N via torchrun).

Workload (default): the ~1M-triangle clutter scene (4,000 seeded objects),
N8L8 BVH from the SAH builder, one frame of 1920x1080 closest-hit primary
rays + 1 any-hit shadow ray per hit + 8 cosine AO rays per hit (length 0.1 x
scene diagonal). A step traces the whole frame (three launches: primary,
shadow, AO) with the rays already resident on the GPU. ``e2e`` is the same
frame through the C-ABI host entry point (bvhgpu_trace_host_batches: the
three batches in one pipelined call) from pinned host buffers, copies
included.

The rays (about 600 MB per frame) are larger than L2; the BVH (~75 MB) stays
resident in L2 across steps, as in steady-state rendering.

``--impl reference`` times the reference's CPU algorithm (the oracle's C
restatement of the ISPC fast path, OpenMP on all host cores) on a bounded
sample of the same frame.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s"

# DRAM bytes per AO ray (dram__bytes_read.sum + dram__bytes_write.sum) of
# this workload's AO call (clutter 4,000 objects, N8L8, FP32 nodes;
# persistent kernel, refill 24, 6 x 10 x 10 direction bins, child-index
# order), from one ncu capture of `bench.py --workload aolaunch --steps 1
# --warmup 1` (2,000,000 AO rays, an evenly strided sample of the frame's):
# the trace kernel 101,412,096 B, the four reorder passes 70,406,912 B. The
# traffic is the ray stream plus the BVH lines that miss L2, so it is scaled
# to a launch by its ray count.
NCU_DRAM_BYTES_PER_AO_RAY = {"trace": 101412096 / 2e6,
                             "with_reorder": (101412096 + 70406912) / 2e6}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--objects", type=int, default=4000)
    p.add_argument("--branching", type=int, default=8)
    p.add_argument("--leaf", type=int, default=8)
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--ao", type=int, default=8)
    p.add_argument("--scheme", default="auto",
                   choices=["auto", "per_ray", "stream", "persistent"])
    p.add_argument("--plan", default="",
                   help="fixed per-batch plan instead of the autotuner: three "
                        "'scheme[,policy,refill,reorder[,any_order]]' specs joined by ';' "
                        "(scheme per_ray_local: per-ray with stacks in local memory)")
    p.add_argument("--nodes", default="fp32", choices=["fp32", "q8"])
    p.add_argument("--top-levels", type=int, default=0)
    p.add_argument("--policy", type=int, default=0, help="persistent: 0 while-while, 1 if-if")
    p.add_argument("--refill", type=int, default=8, help="persistent: idle lanes per refill")
    p.add_argument("--reorder", type=int, default=0,
                   help="fixed scheme: group rays into 6 K^2 direction bins first (0 = off)")
    p.add_argument("--no-compare", action="store_true",
                   help="skip timing the other traversal schemes")
    p.add_argument("--profile", default="instrumented", choices=["instrumented", "fast"])
    p.add_argument("--cpu-sample", type=float, default=0.5,
                   help="fraction of the frame traced by the cpu_baseline leg")
    p.add_argument("--ref-sample", type=float, default=0.1,
                   help="fraction of the frame traced per step by --impl reference")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--report", default="",
                   help="clutter: write the reference's _Info.txt / _Perf.txt and workgroup "
                        "analysis files (whisker plots, _WorkGroupData.txt, "
                        "_WorkGroupUniqueWork.txt) into this folder")
    p.add_argument("--workload", default="clutter",
                   choices=["clutter", "batch64", "adjoint", "scale8m", "terrain", "sweep",
                            "gpuframe", "aolaunch"],
                   help="clutter: the 1M-triangle frame; batch64: 64 scenes in one launch; "
                        "adjoint: forward + backward of the hit distance; scale8m: 8M "
                        "triangles FP32 vs Q8 nodes; terrain: the 32k-triangle terrain, N4L4, "
                        "512x512 + shadow rays; sweep: the clutter frame for every N, L in "
                        "{4,8,12,16}^2, per-ray vs ray-stream; gpuframe: the clutter frame with "
                        "every ray generated on the GPU, AO image read back; aolaunch: the "
                        "clutter frame's AO launch alone on an evenly strided sample of "
                        "--ao-sample rays (the case the ncu DRAM captures profile)")
    p.add_argument("--scenes", type=int, default=64)
    p.add_argument("--job-reorder", type=int, default=8,
                   help="batch64: direction bins per cube face side for the AO jobs (0 = off)")
    p.add_argument("--job-refill", type=int, default=24, help="batch64: refill threshold")
    p.add_argument("--job-any-order", type=int, default=1,
                   help="batch64: child-index push order for the AO jobs (1) or the "
                        "reference's order (0)")
    p.add_argument("--ao-sample", type=int, default=2_000_000,
                   help="aolaunch: AO rays traced per launch (strided sample of the frame's)")
    p.add_argument("--tune-nl", action="store_true",
                   help="batch64: let the autotuner pick N/L per scene, timing each scene's "
                        "jobs in the multi-scene launch itself")
    return p.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def workload_name(a):
    return (f"clutter-{a.objects}obj N{a.branching}L{a.leaf} {a.width}x{a.height} primary "
            f"+1 shadow +{a.ao} AO per hit")


def make_frame(a, scene_trace=None):
    """Triangles, BVH and the three ray batches of one frame. The secondary
    rays come from the primary hits (traced by ``scene_trace``)."""
    import bvhraytracer_gb300 as pkg
    from bvhraytracer_gb300 import scenes as S
    tris = S.clutter(a.objects, seed=1)
    bvh = pkg.Bvh(tris, a.branching, a.leaf)
    primary = S.clutter_camera(a.objects, a.width, a.height)
    return tris, bvh, primary


def secondaries(a, tris, primary, prims):
    from bvhraytracer_gb300 import scenes as S
    m, p, n = S.surface(tris, primary, prims)
    _, _, light = S.clutter_viewpoints(a.objects, seed=1)
    shadow = S.shadow_rays(p, n, light)
    ao = S.ao_rays(p, n, a.ao, 0.1 * S.scene_diagonal(tris), seed=11)
    return shadow, ao


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None
        self.before = 0  # samples taken before the timed region

    def _lines(self):
        try:
            return Path(self.path).read_text().count("\n")
        except OSError:
            return 0

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        # Wait (at most 5 s) for the first sample, so that the sampler runs
        # before the timed region starts; the samples taken until then are
        # left out of the summary when later ones exist.
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None and self._lines() == 0:
            time.sleep(0.005)
        self.before = self._lines()
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        if len(rows) > self.before:
            rows = rows[self.before:]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def sample_packets(rays: np.ndarray, frac: float, packet: int = 256) -> np.ndarray:
    """Every k-th packet of ``packet`` consecutive rays (k = 1/frac), so the
    sample spans the whole frame."""
    k = max(1, int(round(1.0 / frac)))
    npk = -(-rays.shape[0] // packet)
    idx = np.concatenate([np.arange(p * packet, min((p + 1) * packet, rays.shape[0]))
                          for p in range(0, npk, k)])
    return rays[idx]


def cpu_baseline(a, tris, bvh, primary, shadow, ao, frac, repeats=5):
    """The restatement of the reference's ISPC fast path
    (intersectWideAlternative / intersectSecondaryWideAlternative, 16x16
    workgroups, OpenMP dynamic scheduling) with the ISPC kernels' gang lanes
    as 4-wide vectors (oracle/_build/libcpubaseline.so, -O3), on a sample of
    the frame."""
    from oracle import oracle as O
    cv = O.CompactView(bvh.export_compact())
    fv = O.FastView(bvh.export_fast(gang=4))
    parts = [(primary, False), (shadow, True), (ao, True)]
    sample = [(sample_packets(r, frac), any_hit) for r, any_hit in parts]
    n = sum(s.shape[0] for s, _ in sample)
    cores = os.cpu_count() or 1

    def once():
        t0 = time.perf_counter()
        for r, any_hit in sample:
            O.trace_fast(fv, cv, r, any_hit, packet=256, threads=cores, counters=False,
                         outputs=True, baseline=True)
        return time.perf_counter() - t0

    once()  # warm-up, like the reference's first render
    ts = [once() for _ in range(repeats)]
    med = statistics.median(ts)
    return {"value": n / med / 1e6, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{n} rays (every {int(round(1 / frac))}th 256-ray packet of each batch "
                      "of the frame), fast profile (ISPC kernels with 4-wide vector gang lanes, "
                      f"-O3), ray-stream 16x16 packets, median of {repeats} after 1 warm-up",
            "seconds": med}


def oracle_check(a, bvh, batches, device_outs, host_outs, rays_per_batch=24_000):
    """CPU-baseline leg, checking results: an evenly strided sample of each
    timed batch (primary hits, shadow and AO occlusion, as the timed device
    launches and the host entry point left them) against the oracle's
    restatement of the reference on the same rays (instrumented profile:
    CompactNodeManager::intersectImmediately; fast profile:
    FastNodeManager::intersect / intersectSecondary). Returns per batch
    whether both result sets equal the oracle bit for bit."""
    from oracle import oracle as O
    cv = O.CompactView(bvh.export_compact())
    fv = O.FastView(bvh.export_fast(gang=4)) if a.profile == "fast" else None
    res = {}
    for name, (rays, kind), dev_out, host_out in zip(("primary", "shadow", "AO"), batches,
                                                      device_outs, host_outs):
        idx = np.unique(np.linspace(0, rays.shape[0] - 1, rays_per_batch).astype(np.int64))
        any_hit = kind == "any"
        if fv is not None:
            ref = O.trace_fast(fv, cv, rays[idx], any_hit, counters=False)
        else:
            ref = O.trace_instrumented(cv, rays[idx], shadow=any_hit, counters=False)
        want = ref["occluded"] if any_hit else ref["hits"].view(np.uint32)
        got = [np.ascontiguousarray(o[idx]) for o in (dev_out, host_out)]
        if not any_hit:
            got = [g.view(np.uint32) for g in got]
        res[name] = bool(all(np.array_equal(g, want) for g in got))
    res["rays_checked_per_batch"] = int(min(rays_per_batch, min(r.shape[0] for r, _ in batches)))
    res["oracle"] = ("fast profile restatement (FastNodeManager::intersect / "
                     "intersectSecondary)" if fv is not None else
                     "instrumented restatement (CompactNodeManager::intersectImmediately)")
    return res


def run_reference(a):
    """The reference's CPU path (the restated ISPC fast path, vectorised,
    OpenMP on every host core) on a bounded sample of the frame. Nothing of
    the product library runs here: the tree comes from the oracle's C
    restatement of the reference's SAH builder (oracle/sah_builder.c) and the
    FastNodeManager arrays from the oracle's restatement of its constructor;
    the scene and rays come from the numpy generators of
    bvhraytracer_gb300.scenes."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from bvhraytracer_gb300 import scenes as S  # numpy scene generators only
    from oracle import oracle as O
    tris = S.clutter(a.objects, seed=1)
    primary = S.clutter_camera(a.objects, a.width, a.height)
    tree = O.build_tree(tris, a.branching, a.leaf)
    cv = O.CompactView(tree)
    fv = O.FastView(O.fast_arrays(tree, gang=4))
    # Secondary rays from the oracle's own primary hits on the sample.
    frac = a.ref_sample
    ps = sample_packets(primary, frac)
    hits = O.trace_fast(fv, cv, ps, False, packet=256, counters=False, baseline=True)["hits"]
    prims = hits.view(np.int32)[:, 0]
    shadow, ao = secondaries(a, tris, ps, prims)
    sample = [(ps, False), (shadow, True), (ao, True)]
    n = sum(s.shape[0] for s, _ in sample)
    cores = os.cpu_count() or 1

    def step():
        t0 = time.perf_counter()
        for r, any_hit in sample:
            O.trace_fast(fv, cv, r, any_hit, packet=256, threads=cores, counters=False,
                         baseline=True)
        return time.perf_counter() - t0

    for _ in range(a.warmup):
        step()
    ts = [step() for _ in range(a.steps)]
    total = sum(ts)
    value = n * a.steps / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": total / a.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded clutter scene; reference scenes not available)",
        "config": {"workload": workload_name(a), "sample": f"{n} rays per step (every "
                   f"{int(round(1 / frac))}th 256-ray packet of the frame's primary rays and "
                   "their secondaries)", "profile": "fast",
                   "scheme": "ray-stream 16x16 packets",
                   "kernels": "ISPC kernels restated with 4-wide vector gang lanes, -O3 "
                              "(oracle/_build/libcpubaseline.so)",
                   "tree": "oracle/sah_builder.c (the reference's SAH builder restated in C)"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": f"{n} rays per step"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(a):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import bvhraytracer_gb300 as pkg
    from bvhraytracer_gb300 import autotune

    t_setup = time.time()
    tris, bvh, primary = make_frame(a)
    plain = pkg.Scene(bvh, device=local)
    d_primary = torch.from_numpy(primary).to(dev)
    hits0 = plain.trace(d_primary, profile=a.profile)["hits"]
    prims = pkg.hit_prims(hits0.cpu().numpy())
    shadow, ao = secondaries(a, tris, primary, prims)
    d_shadow = torch.from_numpy(shadow).to(dev)
    d_ao = torch.from_numpy(ao).to(dev)
    n_rays = primary.shape[0] + shadow.shape[0] + ao.shape[0]
    out_h = torch.empty((primary.shape[0], 4), dtype=torch.float32, device=dev)
    out_s = torch.empty(shadow.shape[0], dtype=torch.uint8, device=dev)
    out_a = torch.empty(ao.shape[0], dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    batches = [(d_primary, "closest", out_h), (d_shadow, "any", out_s), (d_ao, "any", out_a)]
    names = ["primary (closest)", "shadow (any)", "AO (any)"]

    # Per-batch configuration: the autotuner's choice, or one fixed scheme.
    if a.plan:
        # A fixed per-batch plan, e.g. the autotuner's usual choice, so that a
        # profiler run (whose serialisation skews the autotuner's timings)
        # traces the same launches: "scheme[,policy,refill,reorder[,any_order]]"
        # per batch.
        chosen = []
        for spec in a.plan.split(";"):
            f = spec.split(",")
            o = {"scheme": f[0]}
            if f[0] == "per_ray_local":  # per-ray scheme, stacks in local memory
                o = {"scheme": "per_ray", "stack": "local"}
            if len(f) > 1:
                o.update(policy=int(f[1]), refill=int(f[2]))
            if len(f) > 3 and int(f[3]):
                o["reorder"] = int(f[3])
            if len(f) > 4 and int(f[4]):
                o["any_order"] = True
            chosen.append((plain, o))
        if len(chosen) != 3:
            raise SystemExit("--plan needs three batch specs (primary;shadow;AO)")
        method = f"fixed plan {a.plan}"
        plan_desc = [dict(o, layout="fp32/top0") for _, o in chosen]
    elif a.scheme == "auto":
        plan, scenes = autotune.tune_scene(bvh, [(r, k) for r, k, _ in batches],
                                           profile=a.profile, reps=2, device=local,
                                           scenes={("fp32", 0): plain})
        chosen = [(scenes[lay], dict(opts)) for lay, opts, _ in plan.choices]
        method = "autotuned per batch: " + "; ".join(
            f"{n}: {d['layout']} {d['scheme']}" for n, d in zip(names, plan.describe()))
        plan_desc = plan.describe()
    else:
        sc = plain if (a.nodes == "fp32" and a.top_levels == 0) else pkg.Scene(
            bvh, node_format=a.nodes, top_levels=a.top_levels, device=local)
        o = {"scheme": a.scheme}
        if a.scheme == "persistent":
            o.update(policy=a.policy, refill=a.refill)
        if a.reorder:
            o["reorder"] = a.reorder
        chosen = [(sc, o)] * 3
        method = f"{a.scheme} kernel, {a.nodes} nodes, top levels {a.top_levels}"
        plan_desc = None

    def step(events=None, cfg=None):
        cfg = cfg or chosen
        for i, ((r, kind, out), (sc, o)) in enumerate(zip(batches, cfg)):
            if events is not None:
                events[i][0].record(stream)
            sc.trace(r, kind=kind, out=out, profile=a.profile, **o)
            if events is not None:
                events[i][1].record(stream)

    def frame_ms(cfg, reps=3):
        step(None, cfg)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            step(None, cfg)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps

    # Algorithmic bytes per launch from one counting pass (untimed):
    # node visits x node record bytes + triangle tests x 36 bytes.
    alg = []
    stats = []
    for (r, kind, _), (sc, o) in zip(batches, chosen):
        c = sc.trace(r, kind=kind, counters=True, depth_hist=bool(a.report), profile=a.profile,
                     **o)
        cs = c["counters"].to(torch.int64).sum(0).cpu().numpy()
        if a.report:
            from bvhraytracer_gb300 import report
            stats.append(report.RayStats.from_trace(c["counters"], c["depth_hist"],
                                                    fullness=c["fullness"]))
        alg.append({"node_visits": int(cs[0]), "leaf_visits": int(cs[1]), "tri_tests": int(cs[4]),
                    "bytes": int(cs[0]) * sc.node_record_bytes + int(cs[4]) * 36})
    for sc, _ in chosen:
        sc.status()
    if a.report and rank == 0:
        # The reference's _Info.txt (primary rays; secondary = shadow + AO).
        from bvhraytracer_gb300 import report
        sec = report.RayStats(
            stats[1].rays + stats[2].rays,
            *[getattr(stats[1], k) + getattr(stats[2], k) for k in
              ("node_visits", "leaf_visits", "box_tests", "box_hits", "tri_tests", "tri_hits")],
            stats[1].node_depth + stats[2].node_depth, stats[1].leaf_depth + stats[2].leaf_depth)
        report.write_info(a.report, f"clutter{a.objects}", f"_b{a.branching}_l{a.leaf}",
                          a.branching, a.leaf, stats[0], sec)
        # Workgroup analysis (CameraData::workGroupAnalysisPerImage) of the
        # ray-stream scheme over 16 x 16 packets: primary and shadow rays.
        sh_px = d_shadow  # one shadow ray per pixel, inactive where the primary missed
        if d_shadow.shape[0] != d_primary.shape[0]:
            hit_px = torch.from_numpy(pkg.hit_prims(hits0.cpu().numpy()) >= 0).to(dev)
            sh_px = torch.full_like(d_primary, float("nan"))
            sh_px[hit_px] = d_shadow
        wg_name, wg_problem = f"clutter{a.objects}", f"_b{a.branching}_l{a.leaf}"
        for version in (1, 0):  # intersectWideAlternative, intersectWide
            logs = []
            for r, kind in ((d_primary, "closest"), (sh_px, "any")):
                cap = 1024
                while True:
                    t = plain.trace(r, kind=kind, scheme="stream", counters=True, steps=cap,
                                    wide_alternative=bool(version), profile=a.profile)
                    need = int(t["step_count"].max().item())
                    if need <= cap:
                        break
                    cap = need
                logs.append(t)
            n_groups = (a.width // 16) * (a.height // 16)
            report.write_workgroup_whisker(
                a.report, wg_name, wg_problem, "", 16, version,
                (logs[0]["step_stats"], logs[0]["step_count"]),
                (logs[1]["step_stats"], logs[1]["step_count"]), n_groups)
            report.write_workgroup_data(a.report, wg_name, wg_problem, "", 16, version,
                                        (a.width // 16) * (a.height // 16),
                                        logs[0]["step_stats"], logs[0]["step_count"],
                                        logs[1]["step_stats"], logs[1]["step_count"],
                                        logs[0]["counters"], logs[1]["counters"])
    setup_s = time.time() - t_setup

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    ev = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
           for _ in batches] for _ in range(a.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(dev)
        start.record(stream)
        for k in range(a.steps):
            step(ev[k])
        stop.record(stream)
        torch.cuda.synchronize(dev)
    ms = start.elapsed_time(stop)
    clocks = clk.summary()
    for sc, _ in chosen:
        sc.status()
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    per_kernel_ms = [statistics.mean(e[i][0].elapsed_time(e[i][1]) for e in ev)
                     for i in range(len(batches))]
    value = n_rays * world * a.steps / (ms / 1e3) / 1e6
    ok = torch.equal(out_h.view(torch.int32), hits0.view(torch.int32))

    # End to end through the C-ABI host entry point, pinned host buffers.
    h_rays = [torch.from_numpy(x).pin_memory() for x in (primary, shadow, ao)]
    h_out = [torch.empty((primary.shape[0], 4), dtype=torch.float32).pin_memory(),
             torch.empty(shadow.shape[0], dtype=torch.uint8).pin_memory(),
             torch.empty(ao.shape[0], dtype=torch.uint8).pin_memory()]
    kinds = ["closest", "any", "any"]

    def e2e_step():
        # One bvhgpu_trace_host_batches call per scene layout of the plan
        # (normally one: all three batches in one pipeline).
        groups = {}
        for r, o_buf, kind, (sc, o) in zip(h_rays, h_out, kinds, chosen):
            groups.setdefault(id(sc), (sc, []))[1].append((r.numpy(), kind, o_buf.numpy(), o))
        for sc, items in groups.values():
            sc.trace_host_batches(items, profile=a.profile, stream=stream)

    for _ in range(max(1, a.warmup)):
        e2e_step()
    torch.cuda.synchronize(dev)
    # Each call returns with its results in host memory (it synchronises the
    # stream), so every step is timed on its own: the value is the median
    # step, which a single step slowed by another process on the host's
    # memory does not move; the mean is reported beside it.
    e2e_times = []
    for _ in range(max(3, a.steps)):
        t0 = time.perf_counter()
        e2e_step()
        torch.cuda.synchronize(dev)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_times)
    e2e_mean_s = statistics.mean(e2e_times)
    if world > 1:
        import torch.distributed as dist
        te = torch.tensor([e2e_s, e2e_mean_s], dtype=torch.float64, device=dev)
        dist.all_reduce(te, op=dist.ReduceOp.MAX)  # the slowest rank sets both
        e2e_s, e2e_mean_s = (float(x) for x in te.tolist())
    e2e_ok = (np.array_equal(h_out[0].numpy().view(np.uint32), out_h.cpu().numpy().view(np.uint32))
              and np.array_equal(h_out[2].numpy(), out_a.cpu().numpy()))
    h2d = sum(x.numel() * 4 for x in h_rays)
    d2h = sum(x.numel() * x.element_size() for x in h_out)

    # Roofline of the dominant kernel (largest share of the step).
    dom = int(np.argmax(per_kernel_ms))
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg[dom]["bytes"] / (per_kernel_ms[dom] / 1e3) / 1e9
    # The BVH (nodes + leaves) fits the 129 MB L2, so the bound that applies
    # is L2's read rate: measured here with the library's streaming read
    # kernel over a 60 MB buffer (median of 7, 20 passes each).
    l2_peak = pkg.read_bandwidth(60 << 20, device=local)
    traffic = None
    dom_opts = chosen[dom][1]
    if (names[dom].startswith("AO") and dom_opts.get("scheme") == "persistent"
            and dom_opts.get("reorder") == 10 and chosen[dom][0].node_format == "fp32"
            and a.objects == 4000 and a.branching == 8 and a.leaf == 8):
        traffic = NCU_DRAM_BYTES_PER_AO_RAY["with_reorder"] * int(batches[dom][0].shape[0])

    compare = {}
    if not a.no_compare:
        plain_cfg = [(plain, {"scheme": "per_ray"})] * 3
        compare["plain_per_ray_fp32"] = frame_ms(plain_cfg)
        compare["stream_fp32_wg16"] = frame_ms([(plain, {"scheme": "stream"})] * 3)
        compare["persistent_fp32"] = frame_ms([(plain, {"scheme": "persistent"})] * 3)
        compare["this_method"] = ms / a.steps
        compare["speedup_vs_plain_per_ray"] = compare["plain_per_ray_fp32"] / (ms / a.steps)
    cpu = parity = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu = cpu_baseline(a, tris, bvh, primary, shadow, ao, a.cpu_sample)
        parity = oracle_check(a, bvh, ((primary, "closest"), (shadow, "any"), (ao, "any")),
                              [x.cpu().numpy() for x in (out_h, out_s, out_a)],
                              [x.numpy() for x in h_out])

    if a.report and rank == 0:
        from bvhraytracer_gb300 import report
        cx = bvh.export_compact()
        leaves = cx["child_count"] == 0
        report.write_perf(a.report, f"clutter{a.objects}", f"_b{a.branching}_l{a.leaf}"
                          f"_mb{a.branching}_ml{a.leaf}", a.branching, a.leaf, 4,
                          -(-a.branching // 4) * 4, -(-a.leaf // 4) * 4, ms / a.steps / 1e3,
                          float(cx["depth"][leaves].mean()), int(bvh.info["n_tris"]))
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded clutter scene standing in for the reference's glTF scenes)",
            "config": {
                "workload": workload_name(a), "method": method, "plan": plan_desc,
                "profile": a.profile, "triangles": int(bvh.info["n_tris"]),
                "rays_per_step": n_rays, "primary": int(primary.shape[0]),
                "shadow": int(shadow.shape[0]), "ao": int(ao.shape[0]),
                "results_equal_plain_kernel": bool(ok),
                "oracle_equal": parity,
                "l2": "inputs larger than L2 (rays ~%d MB per step); BVH stays L2-resident"
                      % (n_rays * 32 // 2**20),
                # beside the records: one 4-byte stack entry per child slot and
                # 6 of the leaf block's 9 floats per triangle slot (bounds)
                "bvh_bytes": {"nodes_fp32": plain.node_bytes, "leaves": plain.leaf_bytes,
                              "child_entries": plain.node_bytes // plain.node_record_bytes
                              * (-(-a.branching // 4) * 4) * 4,
                              "triangle_bounds": plain.leaf_bytes * 6 // 9},
                "per_kernel_ms": dict(zip(names, per_kernel_ms)),
                "ms_per_frame_by_method": compare,
                "setup_s": round(setup_s, 2),
            },
            "roofline": {
                "bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks
                else "fallback",
                "traffic": traffic,
                "traffic_source": ("ncu DRAM bytes per AO ray of the same scene's AO call "
                                   "(trace kernel + reorder passes), captured on a 2M-ray "
                                   "strided sample and scaled by rays" if traffic else None),
                "algorithmic_bytes_per_launch": alg[dom]["bytes"],
                "bytes_rule": "node visits x node record bytes + triangle tests x 36 B",
                "l2_peak": l2_peak, "l2_frac": achieved / l2_peak,
                "l2_peak_source": "measured: bvhgpu_read_bandwidth, 60 MB buffer read 20 times "
                                  "per launch, L1 bypassed, median of 7",
            },
            "e2e": {"value": n_rays * world / e2e_s / 1e6, "unit": METRIC,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "statistic": f"median of {len(e2e_times)} steps",
                    "mean_value": n_rays * world / e2e_mean_s / 1e6,
                    "step_ms": [round(x * 1e3, 3) for x in e2e_times],
                    "matches_device_results": bool(e2e_ok)},
            "cpu_baseline": cpu,
            "clocks": clocks,
            # per trace call: one traversal launch, plus four reorder passes
            # (bin, scan, scan, scatter) when the plan groups the rays first
            "gpu_launches": sum(1 + (4 if o.get("reorder") else 0) for _, o in chosen) * a.steps,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def batch_scenes(a, seed=5):
    """Scene and ray specs of the multi-scene workload: triangle counts
    log-uniform in 1k..500k, ray counts log-uniform in 4k..2M split 1:1:4
    between primary, shadow and AO rays; terrain and clutter alternate."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(a.scenes):
        t = float(np.exp(rng.uniform(np.log(1e3), np.log(5e5))))
        r = float(np.exp(rng.uniform(np.log(4e3), np.log(2e6))))
        specs.append(("terrain" if i % 2 == 0 else "clutter", t, r, i))
    return specs


def make_batch_scene(kind, tris_target, rays_target, i):
    from bvhraytracer_gb300 import scenes as S
    n_primary = max(64, int(rays_target / 6))
    w = max(8, int(round(np.sqrt(n_primary * 16 / 9))))
    h = max(8, n_primary // w)
    if kind == "terrain":
        n = max(4, int(round(np.sqrt(tris_target / 2))))
        tris = S.terrain(n, seed=100 + i)
        c = np.array([0.5, 0.0, 0.5])
        primary = S.camera_rays(c + [0.0, 0.7, 0.9], c, w, h)
        light = np.array([2.0, 3.0, 2.0], np.float32)
    else:
        n_obj = max(1, int(round(tris_target / 250)))
        tris = S.clutter(n_obj, seed=100 + i)
        cam, target, light = S.clutter_viewpoints(n_obj, seed=100 + i)
        primary = S.camera_rays(cam, target, w, h)
    return tris, primary, light


def run_batch(a):
    """Many scenes of uneven size and ray count in one persistent launch
    (recorded in a CUDA graph) against one plain per-ray launch per batch."""
    import torch
    import bvhraytracer_gb300 as pkg
    from bvhraytracer_gb300 import autotune
    from bvhraytracer_gb300 import scenes as S
    dev = torch.device("cuda", 0)
    t_setup = time.time()
    scenes, jobs_plain, chosen, job_reorder = [], [], [], []
    n_tris = n_rays = 0
    for kind, tt, rr, i in batch_scenes(a):
        tris, primary, light = make_batch_scene(kind, tt, rr, i)
        d_p = torch.from_numpy(primary).to(dev)
        if a.tune_nl:
            def batches_fn(scene, d_p=d_p, tris=tris, primary=primary, light=light, i=i):
                h = scene.trace(d_p)["hits"]
                m, p, n = S.surface(tris, primary, pkg.hit_prims(h.cpu().numpy()))
                sh = torch.from_numpy(S.shadow_rays(p, n, light)).to(dev)
                ao = torch.from_numpy(S.ao_rays(p, n, 4, 0.1 * S.scene_diagonal(tris),
                                                seed=i)).to(dev)
                return [(d_p, "closest"), (sh, "any"), (ao, "any")]

            def time_fn(scene, batches):
                # the scene's three jobs in the multi-scene launch itself
                jobs = []
                for (rays, k), (ro, ao_job) in zip(batches, ((0, 0), (0, 0),
                                                             (a.job_reorder, a.job_any_order))):
                    out = (torch.empty((rays.shape[0], 4), dtype=torch.float32, device=dev)
                           if k == "closest" else
                           torch.empty(rays.shape[0], dtype=torch.uint8, device=dev))
                    jobs.append((scene, rays, k, out, ro, ao_job))
                stream = torch.cuda.current_stream(dev)
                pkg.trace_jobs(jobs, policy=2, refill=a.job_refill)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(3):
                    pkg.trace_jobs(jobs, policy=2, refill=a.job_refill)
                e1.record(stream)
                torch.cuda.synchronize(dev)
                return e0.elapsed_time(e1) / 3

            best, _ = autotune.tune_branching(
                tris, batches_fn, pairs=tuple((n, l) for n in (4, 8, 16) for l in (4, 8, 16)),
                layouts=(("fp32", 0),), time_fn=time_fn, reps=1,
                prefer=(a.branching, a.leaf), margin=0.05)
            _, (bn, bl), bvh, plan, tuned = best
            scene = tuned[("fp32", 0)]
            block, stack = 128, "shared"
        else:
            bn, bl, block, stack = a.branching, a.leaf, 128, "shared"
            bvh = pkg.Bvh(tris, bn, bl)
            scene = pkg.Scene(bvh)
        h = scene.trace(d_p)["hits"]
        m, p, n = S.surface(tris, primary, pkg.hit_prims(h.cpu().numpy()))
        sh = torch.from_numpy(S.shadow_rays(p, n, light)).to(dev)
        ao = torch.from_numpy(S.ao_rays(p, n, 4, 0.1 * S.scene_diagonal(tris), seed=i)).to(dev)
        for rays, k, ro, ao_job in ((d_p, "closest", 0, 0), (sh, "any", 0, 0),
                                    (ao, "any", a.job_reorder, a.job_any_order)):
            out = (torch.empty((rays.shape[0], 4), dtype=torch.float32, device=dev)
                   if k == "closest" else torch.empty(rays.shape[0], dtype=torch.uint8, device=dev))
            jobs_plain.append((scene, rays, k, out))
            job_reorder.append((ro, ao_job))
            n_rays += rays.shape[0]
        scenes.append({"kind": kind, "triangles": int(bvh.info["n_tris"]), "N": bn, "L": bl,
                       "block": block, "stack": stack,
                       "rays": int(d_p.shape[0] + sh.shape[0] + ao.shape[0])})
        chosen.append((block, stack))
        n_tris += int(bvh.info["n_tris"])
    setup_s = time.time() - t_setup
    stream = torch.cuda.current_stream(dev)
    blocks = [b for b in chosen for _ in range(3)]

    def sequential():
        for (scene, rays, k, out), (b, st) in zip(jobs_plain, blocks):
            scene.trace(rays, kind=k, scheme="per_ray", block=b, stack=st, out=out)

    # The AO jobs' rays are grouped by direction inside the batched call.
    jobs_batched = [j + x for j, x in zip(jobs_plain, job_reorder)]

    def batched(one_launch=False):
        pkg.trace_jobs(jobs_batched, policy=2, refill=a.job_refill, one_launch=one_launch)

    def timed(fn, steps):
        for _ in range(a.warmup):
            fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / steps

    # Reference results of the sequential plain launches, then the batch.
    sequential()
    refs = [out.clone() for (_, _, _, out) in jobs_plain]
    batched()
    torch.cuda.synchronize(dev)
    same = all(torch.equal(o.view(torch.uint8), r.view(torch.uint8))
               for (_, _, _, o), r in zip(jobs_plain, refs))
    batched(one_launch=True)
    torch.cuda.synchronize(dev)
    same_one = all(torch.equal(o.view(torch.uint8), r.view(torch.uint8))
                   for (_, _, _, o), r in zip(jobs_plain, refs))
    # The batched launches recorded in CUDA graphs: one launch per ray kind
    # (and node width and format), and one launch for everything.
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        batched()
    g1 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g1):
        batched(one_launch=True)
    ms_one = timed(g1.replay, a.steps)
    ms_graph = timed(g.replay, a.steps)
    # The headline takes the faster launch form, timed again with the clock
    # sampler: per-scene N / L choices split the per-kind form into one launch
    # per ray kind and node width, which the single launch does not need.
    one_form = ms_one < ms_graph
    with ClockSampler(0) as clk:
        ms_head = timed(g1.replay if one_form else g.replay, a.steps)
    clocks = clk.summary()
    ms_batched = timed(batched, a.steps)
    per_kind_launches = len({(k, s_.bvh_info["branching"]) for s_, _, k, _ in jobs_plain})
    launches = (1 if one_form else per_kind_launches) + (4 if a.job_reorder else 0)
    ms_seq = timed(sequential, a.steps)
    for s_ in {id(j[0]): j[0] for j in jobs_plain}.values():
        s_.status()
    line = {
        "metric": METRIC, "value": n_rays / (ms_head / 1e3) / 1e6, "unit": METRIC, "n_gpus": 1,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_head, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded terrain and clutter scenes)",
        "config": {
            "workload": f"{a.scenes} scenes in one persistent launch, triangles log-uniform "
                        f"1k-500k, rays log-uniform 4k-2M (primary:shadow:AO 1:1:4)",
            "triangles_total": n_tris, "rays_per_step": n_rays, "jobs": len(jobs_plain),
            "method": "bvhgpu_trace_jobs ("
                      + ("one persistent launch for all jobs, closest-hit rays first"
                         if one_form else
                         f"one persistent launch per ray kind and node width ({per_kind_launches})")
                      + " over all scenes; speculative any-hit policy"
                      + (f", AO jobs grouped into 6x{a.job_reorder}x{a.job_reorder} direction bins"
                         + (", child-index push order" if a.job_any_order else "")
                         if a.job_reorder else "")
                      + ") in a CUDA graph; the faster of the two launch forms",
            "launch_form": "one launch" if one_form else "per ray kind",
            "ms_batched_graph": ms_graph, "ms_batched_no_graph": ms_batched,
            "ms_one_launch_graph": ms_one, "one_launch_results_identical": bool(same_one),
            "ms_sequential_plain_launches": ms_seq,
            "speedup_vs_sequential": ms_seq / ms_head, "results_identical": bool(same),
            "autotuned_nl": bool(a.tune_nl), "scenes": scenes, "setup_s": round(setup_s, 1),
        },
        # per step the batched launch(es) of the chosen form plus the four
        # segmented reorder passes
        "clocks": clocks, "gpu_launches": a.steps * launches,
    }
    print(json.dumps(line))


def fd_check(verts, faces, rays, prim, mask, t_tgt, gv, n_coords=512, seed=3):
    """Central finite differences in FP64 of the fixed-visibility loss on
    sampled vertex coordinates, at h = 1e-4 (truncation-limited on grazing
    rays), 1e-6 and 1e-7, and Richardson-extrapolated from h = 1e-4 and 5e-5;
    and the exact FP64 gradient of the same loss (PyTorch float64 autograd of
    Moller-Trumbore on the CPU, same hit set). Returns the norm-relative error
    of the FP32 adjoint against each, and of each difference quotient against
    the exact FP64 gradient (the truncation error of the differences)."""
    V = verts.astype(np.float64)
    R = rays.astype(np.float64)
    hit = np.nonzero(mask)[0]
    tri_of = prim[hit]
    F = faces
    touched = np.unique(F[tri_of].reshape(-1))
    rng = np.random.default_rng(seed)
    vids = rng.choice(touched, n_coords, replace=len(touched) < n_coords)
    axes = rng.integers(0, 3, n_coords)
    order = np.argsort(tri_of)
    sorted_tris = tri_of[order]
    fd = {h: np.zeros(n_coords) for h in (1e-4, 5e-5, 1e-6, 1e-7)}
    for k, (vid, ax) in enumerate(zip(vids, axes)):
        tris = np.nonzero(np.any(F == vid, axis=1))[0]
        lo = np.searchsorted(sorted_tris, tris, "left")
        hi = np.searchsorted(sorted_tris, tris, "right")
        rr = hit[np.concatenate([order[a:b] for a, b in zip(lo, hi)])]
        tt = F[prim[rr]]
        o, d = R[rr, 0:3], R[rr, 4:7]
        p0b, p1b, p2b = V[tt[:, 0]], V[tt[:, 1]], V[tt[:, 2]]

        def L(delta):
            p0, p1, p2 = p0b.copy(), p1b.copy(), p2b.copy()
            p0[tt[:, 0] == vid, ax] += delta
            p1[tt[:, 1] == vid, ax] += delta
            p2[tt[:, 2] == vid, ax] += delta
            e1, e2 = p1 - p0, p2 - p0
            s1 = np.cross(d, e2)
            inv = 1.0 / np.sum(s1 * e1, -1)
            s2 = np.cross(o - p0, e1)
            t = np.sum(e2 * s2, -1) * inv
            return np.sum((t - t_tgt[rr]) ** 2)
        for h in fd:
            fd[h][k] = (L(h) - L(-h)) / (2 * h)
    ad = gv[vids, axes].astype(np.float64)
    import torch
    from bvhraytracer_gb300 import diff as D
    Vt = torch.from_numpy(V).requires_grad_(True)
    Rt = torch.from_numpy(R[hit])
    Ft = torch.from_numpy(F[tri_of].astype(np.int64))
    t64, _, _ = D.moller_trumbore_torch(Rt[:, 0:3], Rt[:, 4:7], Vt[Ft[:, 0]], Vt[Ft[:, 1]],
                                        Vt[Ft[:, 2]])
    g64, = torch.autograd.grad(((t64 - torch.from_numpy(t_tgt[hit])) ** 2).sum(), (Vt,))
    exact = g64.numpy()[vids, axes]

    def rel(x, ref=None):
        y = ad if ref is None else ref
        return float(np.linalg.norm(y - x) / max(np.linalg.norm(x), 1e-300))
    rich = (4 * fd[5e-5] - fd[1e-4]) / 3
    return {"h=1e-4": rel(fd[1e-4]), "h=1e-6": rel(fd[1e-6]), "h=1e-7": rel(fd[1e-7]),
            "richardson(1e-4, 5e-5)": rel(rich), "fp64_autograd": rel(exact),
            "fd_truncation_vs_fp64_autograd": {
                "h=1e-4": rel(exact, fd[1e-4]), "h=1e-6": rel(exact, fd[1e-6]),
                "h=1e-7": rel(exact, fd[1e-7]), "richardson(1e-4, 5e-5)": rel(exact, rich)}}


def run_adjoint(a):
    """Forward + backward of sum over 1M primary rays of (t - t_target)^2,
    t_target from vertices moved by seeded N(0, 0.01) noise; terrain
    256 x 256 quads and the 1M-triangle clutter scene."""
    import torch
    from bvhraytracer_gb300 import diff as D
    from bvhraytracer_gb300 import scenes as S
    dev = torch.device("cuda", 0)
    results = {}
    rng = np.random.default_rng(11)
    for name in ("terrain256", "clutter1M"):
        if name == "terrain256":
            verts, faces = S.terrain_mesh(256, seed=0)
            c = np.array([0.5, 0.0, 0.5])
            rays = S.camera_rays(c + [0.0, 0.55, 0.65], c, 1024, 1024)
        else:
            tris = S.clutter(a.objects, seed=1)
            verts = tris.reshape(-1, 3)
            faces = np.arange(verts.shape[0], dtype=np.int64).reshape(-1, 3)
            cam, target, _ = S.clutter_viewpoints(a.objects, seed=1)
            rays = S.camera_rays(cam, target, 1024, 1024)
        v = torch.from_numpy(verts).to(dev).requires_grad_(True)
        f = torch.from_numpy(faces.astype(np.int32)).to(dev)  # int32: no per-step conversion
        r = torch.from_numpy(rays).to(dev).requires_grad_(True)
        scene = D.scene_for(v, f)
        vt = torch.from_numpy(verts + rng.normal(0, 0.01, verts.shape).astype(np.float32)).to(dev)
        t_tgt, _, _, p_tgt = D.ray_hit(vt, f, r.detach(), D.scene_for(vt, f))

        def step(recompute=False):
            t, u, w, prim = D.ray_hit(v, f, r, scene, recompute=recompute)
            m = (prim >= 0) & (p_tgt >= 0)
            # masked by multiplication (no boolean indexing, so no host sync)
            loss = torch.where(m, (t - t_tgt) ** 2, torch.zeros_like(t)).sum()
            gv, gr = torch.autograd.grad(loss, (v, r))
            return loss, gv, gr, prim, m

        stream = torch.cuda.current_stream(dev)

        def timed(recompute):
            for _ in range(a.warmup):
                step(recompute)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(a.steps):
                res = step(recompute)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            return e0.elapsed_time(e1) / a.steps, res

        # the backward re-tracing each ray instead of reading the stored hits
        ms_re, _ = timed(True)
        ms, (loss, gv, gr, prim, m) = timed(False)
        fdr = fd_check(verts, faces, rays, prim.cpu().numpy(), m.cpu().numpy(),
                       t_tgt.cpu().numpy().astype(np.float64), gv.cpu().numpy())
        scene.status()
        results[name] = {"triangles": int(faces.shape[0]), "rays": int(rays.shape[0]),
                         "hits": int(m.sum().item()), "ms_forward_backward": ms,
                         "mrays_per_s_forward_backward": rays.shape[0] / (ms / 1e3) / 1e6,
                         "ms_forward_backward_recompute": ms_re,
                         "fd_fp64_norm_relative_error": fdr,
                         "fd": "central, FP64, 512 sampled vertex coordinates"}
    line = {
        "metric": "Mrays/s (forward+backward)",
        "value": results["clutter1M"]["mrays_per_s_forward_backward"],
        "unit": "Mrays/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": results["clutter1M"]["ms_forward_backward"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded terrain and clutter scenes)",
        "config": {"workload": "adjoint: loss sum (t - t_target)^2 over 1M primary rays",
                   "results": results},
    }
    print(json.dumps(line))


# DRAM bytes per AO ray of the 8M-triangle scene's AO call (trace kernel +
# the four reorder passes; policy 2, refill 24, 6 x 10 x 10 bins,
# child-index order), from one ncu capture each of `bench.py --workload
# aolaunch --objects 32000 --leaf 4 --ao 16 --steps 1 --warmup 1 [--nodes
# q8]` (2,000,000 strided AO rays): FP32 209,611,008 + 70,400,256 B, Q8
# 190,471,680 + 70,404,864 B.
SCALE8M_DRAM_BYTES_PER_AO_RAY = {"fp32": (209611008 + 70400256) / 2e6,
                                 "q8": (190471680 + 70404864) / 2e6}


def run_scale(a):
    """Clutter scene scaled to ~8M triangles (32,000 objects), N8L4, one frame
    of 1920x1080 primary rays + 16 AO rays per hit: FP32 against Q8 nodes
    (hit sets compared ray by ray), node bytes per ray, algorithmic GB/s, and
    the FP64 error of 1M sampled closest hits."""
    import torch
    import bvhraytracer_gb300 as pkg
    from bvhraytracer_gb300 import scenes as S
    dev = torch.device("cuda", 0)
    pk = ROOT / "MEASURED_PEAKS.json"
    hbm_peak = json.loads(pk.read_text()).get("hbm_gbs", 6800.0) if pk.exists() else 6800.0
    n_obj = 32000
    t0 = time.time()
    tris = S.clutter(n_obj, seed=1)
    bvh = pkg.Bvh(tris, 8, 4)
    build_s = time.time() - t0
    scenes = {"fp32": pkg.Scene(bvh), "q8": pkg.Scene(bvh, node_format="q8")}
    primary = torch.from_numpy(S.clutter_camera(n_obj, 1920, 1080)).to(dev)
    h0 = scenes["fp32"].trace(primary)["hits"]
    prims = pkg.hit_prims(h0.cpu().numpy())
    m, p, n = S.surface(tris, primary.cpu().numpy(), prims)
    ao = torch.from_numpy(S.ao_rays(p, n, 16, 0.1 * S.scene_diagonal(tris), seed=3)).to(dev)
    stream = torch.cuda.current_stream(dev)
    res = {}
    for name, sc in scenes.items():
        best = None
        for o in ({"scheme": "per_ray"}, {"scheme": "persistent", "policy": 0, "refill": 16},
                  {"scheme": "persistent", "policy": 2, "refill": 16},
                  {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10,
                   "any_order": True}):
            outs = []
            ms = []
            for rays, kind in ((primary, "closest"), (ao, "any")):
                sc.trace(rays, kind=kind, **o)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(a.steps):
                    out = sc.trace(rays, kind=kind, **o)
                e1.record(stream)
                torch.cuda.synchronize(dev)
                ms.append(e0.elapsed_time(e1) / a.steps)
                outs.append(out["hits" if kind == "closest" else "occluded"])
            if best is None or sum(ms) < sum(best[1]):
                best = (o, ms, outs)
        o, ms, outs = best
        cnt = [sc.trace(r, kind=k, counters=True, **o)["counters"].to(torch.int64).sum(0).cpu()
               for r, k in ((primary, "closest"), (ao, "any"))]
        bytes_ = [int(c[0]) * sc.node_record_bytes + int(c[4]) * 36 for c in cnt]
        nrays = [primary.shape[0], ao.shape[0]]
        res[name] = {
            "options": o, "ms_primary": ms[0], "ms_ao": ms[1],
            "mrays_per_s": (nrays[0] + nrays[1]) / ((ms[0] + ms[1]) / 1e3) / 1e6,
            "node_record_bytes": sc.node_record_bytes, "node_bytes_total": sc.node_bytes,
            "node_bytes_per_ray": {"primary": int(cnt[0][0]) * sc.node_record_bytes / nrays[0],
                                   "ao": int(cnt[1][0]) * sc.node_record_bytes / nrays[1]},
            "algorithmic_gb_per_s_ao": bytes_[1] / (ms[1] / 1e3) / 1e9,
            "_outs": outs,
        }
        if o.get("reorder") == 10 and o.get("policy") in (2, 3):
            # HBM side of the AO call from measured DRAM bytes per AO ray
            dram = SCALE8M_DRAM_BYTES_PER_AO_RAY[name] * nrays[1]
            res[name]["dram_bytes_per_ao_ray"] = SCALE8M_DRAM_BYTES_PER_AO_RAY[name]
            res[name]["dram_gb_per_s_ao"] = dram / (ms[1] / 1e3) / 1e9
            res[name]["hbm_frac_ao"] = res[name]["dram_gb_per_s_ao"] / hbm_peak
        sc.status()
    same_h = torch.equal(res["q8"]["_outs"][0].view(torch.int32), res["fp32"]["_outs"][0].view(torch.int32))
    same_a = torch.equal(res["q8"]["_outs"][1], res["fp32"]["_outs"][1])
    for r in res.values():
        r.pop("_outs")
    # FP64 error of 1M sampled closest hits.
    idx = torch.randperm(primary.shape[0], generator=torch.Generator().manual_seed(0))[:1000000]
    sample = primary[idx.to(dev)].contiguous()
    hs = scenes["fp32"].trace(sample)["hits"]
    chk = scenes["fp32"].fp64_check(sample, hs).cpu().numpy()
    hv = hs.cpu().numpy()
    ok = ~np.isnan(chk[:, 0])
    err = {"rays": int(ok.sum()), "t_rel_max": float(np.max(chk[ok, 3])),
           "t_rel_median": float(np.median(chk[ok, 3])),
           "b1_abs_max": float(np.max(np.abs(hv[ok, 2] - chk[ok, 1]))),
           "b2_abs_max": float(np.max(np.abs(hv[ok, 3] - chk[ok, 2])))}
    total = primary.shape[0] + ao.shape[0]
    best_name = min(res, key=lambda k: res[k]["ms_primary"] + res[k]["ms_ao"])
    line = {
        "metric": METRIC, "value": res[best_name]["mrays_per_s"], "unit": METRIC, "n_gpus": 1,
        "steps": a.steps, "warmup": 1,
        "ms_per_step": res[best_name]["ms_primary"] + res[best_name]["ms_ao"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded clutter scene, 32,000 objects)",
        "config": {"workload": "clutter-32000obj N8L4 1920x1080 primary + 16 AO per hit",
                   "triangles": int(bvh.info["n_tris"]), "rays_per_step": int(total),
                   "build_s": round(build_s, 1), "by_node_format": res,
                   "q8_hits_identical": bool(same_h), "q8_occlusion_identical": bool(same_a),
                   "fp64_error_1M_sampled_hits": err},
    }
    print(json.dumps(line))


def _time_trace(sc, rays, kind, opts, reps, stream):
    import torch
    sc.trace(rays, kind=kind, **opts)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        out = sc.trace(rays, kind=kind, **opts)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, out


def run_terrain(a):
    """The 128 x 128-quad terrain (32,768 triangles), N4L4, 512 x 512 primary
    rays + 1 shadow ray per hit toward (2, 3, 2): per-ray, ray-stream and
    persistent kernels, results checked against the oracle, and the oracle's
    restatement of the ISPC path on every host core on the whole frame."""
    import torch
    import bvhraytracer_gb300 as pkg
    from bvhraytracer_gb300 import scenes as S
    from oracle import oracle as O
    dev = torch.device("cuda", 0)
    tris, rays, light = S.terrain_workload()
    bvh = pkg.Bvh(tris, 4, 4)
    sc = pkg.Scene(bvh)
    d_p = torch.from_numpy(rays).to(dev)
    cv = O.CompactView(bvh.export_compact())
    ref = O.trace_instrumented(cv, rays, False, counters=False)
    prims = ref["hits"].view(np.int32)[:, 0]
    m, p, n = S.surface(tris, rays, prims)
    shadow = S.shadow_rays(p, n, light)
    d_s = torch.from_numpy(shadow).to(dev)
    ref_s = O.trace_instrumented(cv, shadow, True, counters=False)["occluded"]
    stream = torch.cuda.current_stream(dev)
    res = {}
    for name, o in (("per_ray", {"scheme": "per_ray"}), ("stream_wg16", {"scheme": "stream"}),
                    ("persistent", {"scheme": "persistent", "policy": 0, "refill": 16}),
                    ("per_ray_local", {"scheme": "per_ray", "stack": "local"}),
                    # primary per-ray with local stacks, shadow persistent policy 2
                    ("mixed", [{"scheme": "per_ray", "stack": "local"},
                               {"scheme": "persistent", "policy": 2, "refill": 16}])):
        op, os_ = (o[0], o[1]) if isinstance(o, list) else (o, o)
        ms_p, hp = _time_trace(sc, d_p, "closest", op, a.steps, stream)
        ms_s, hs = _time_trace(sc, d_s, "any", os_, a.steps, stream)
        ok = (np.array_equal(hp["hits"].cpu().numpy().view(np.uint32), ref["hits"].view(np.uint32))
              and np.array_equal(hs["occluded"].cpu().numpy(), ref_s))
        res[name] = {"ms_primary": ms_p, "ms_shadow": ms_s,
                     "mrays_per_s": (rays.shape[0] + shadow.shape[0]) / ((ms_p + ms_s) / 1e3) / 1e6,
                     "equal_to_oracle": bool(ok)}
    sc.status()
    fv = O.FastView(bvh.export_fast(gang=4))
    cores = os.cpu_count() or 1

    def cpu_once():
        t0 = time.perf_counter()
        O.trace_fast(fv, cv, rays, False, packet=256, threads=cores, counters=False)
        O.trace_fast(fv, cv, shadow, True, packet=256, threads=cores, counters=False)
        return time.perf_counter() - t0
    cpu_once()
    cpu_s = statistics.median([cpu_once() for _ in range(5)])
    best = max(res, key=lambda k: res[k]["mrays_per_s"])
    total = rays.shape[0] + shadow.shape[0]
    line = {
        "metric": METRIC, "value": res[best]["mrays_per_s"], "unit": METRIC, "n_gpus": 1,
        "steps": a.steps, "warmup": 1,
        "ms_per_step": res[best]["ms_primary"] + res[best]["ms_shadow"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded sine-octave terrain)",
        "config": {"workload": "terrain 128x128 quads (32,768 triangles) N4L4, 512x512 primary "
                               "+ 1 shadow per hit", "rays_per_step": int(total),
                   "by_scheme": res, "best": best,
                   "l2": "scene and rays (10 MB) fit in L2: a small, cache-resident case"},
        "cpu_baseline": {"value": total / cpu_s / 1e6, "unit": METRIC, "cores": cores,
                         "kind": "port", "sample": "the whole frame, fast profile, ray-stream "
                         "16x16 packets, median of 5 after 1 warm-up"},
    }
    print(json.dumps(line))


def run_gpuframe(a):
    """The clutter frame rendered on the GPU end to end: camera rays
    (bvhgpu_camera_rays), primary closest hits, shadow and 8 cosine AO rays
    per hit generated from the hits (bvhgpu_secondary_rays), the shadow and
    AO traces, and the per-pixel AO factor (bvhgpu_ao_factor); the AO image
    is read back to the host each step. No rays cross the host boundary."""
    import torch
    import bvhraytracer_gb300 as pkg
    from bvhraytracer_gb300 import scenes as S
    from oracle import oracle as O
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    t_setup = time.time()
    tris = S.clutter(a.objects, seed=1)
    bvh = pkg.Bvh(tris, a.branching, a.leaf)
    sc = pkg.Scene(bvh)
    cam, target, light = S.clutter_viewpoints(a.objects, seed=1)
    ao_len = float(0.1 * S.scene_diagonal(tris))
    w, h, spp = a.width, a.height, a.ao
    img = torch.empty(w * h, dtype=torch.float32).pin_memory()

    def frame():
        prim = pkg.camera_rays(cam, target, w, h)
        hits = sc.trace(prim, scheme="per_ray", stack="local")["hits"]
        sh, ao = sc.secondary_rays(prim, hits, light=light, ao_samples=spp, ao_length=ao_len,
                                   sampling="cosine", seed=0)
        occ_s = sc.trace(sh, kind="any", scheme="persistent", policy=2, refill=16)["occluded"]
        occ_a = sc.trace(ao, kind="any", scheme="persistent", policy=2, refill=24, reorder=10,
                         any_order=True)["occluded"]
        return prim, hits, sh, ao, occ_s, occ_a, pkg.ao_factor(occ_a, spp)

    prim, hits, sh, ao, occ_s, occ_a, fac = frame()
    torch.cuda.synchronize(dev)
    setup_s = time.time() - t_setup
    active = lambda r: int((~torch.isnan(r[:, 0])).sum().item())
    n_prim, n_sh, n_ao = prim.shape[0], active(sh), active(ao)
    n_rays = n_prim + n_sh + n_ao
    # Parity on samples of the GPU-made rays: the oracle traces the same rays.
    cv = O.CompactView(bvh.export_compact())
    rng = np.random.default_rng(5)
    checks = {}
    for name, rays, kind, out in (("primary", prim, "closest", hits), ("shadow", sh, "any", occ_s),
                                  ("ao", ao, "any", occ_a)):
        idx = np.sort(rng.choice(rays.shape[0], min(20000, rays.shape[0]), replace=False))
        r = rays.cpu().numpy()[idx]
        ref = O.trace_instrumented(cv, r, shadow=kind == "any", counters=False)
        got = out.cpu().numpy()[idx]
        want = ref["hits"] if kind == "closest" else ref["occluded"]
        checks[name] = bool(np.array_equal(got.view(np.uint8), want.view(np.uint8)))
    sc.status()

    def timed(fn):
        for _ in range(a.warmup):
            fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / a.steps

    ms_eager = timed(frame)
    outs = {}

    def capture_body():
        outs["f"] = frame()[-1]
    capture_body()
    torch.cuda.synchronize(dev)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        capture_body()
    with ClockSampler(0) as clk:
        ms_graph = timed(g.replay)
    clocks = clk.summary()
    graph_ok = bool(torch.equal(outs["f"], fac))

    def e2e_step():
        g.replay()
        img.copy_(outs["f"], non_blocking=True)
        torch.cuda.synchronize(dev)
    for _ in range(a.warmup):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / a.steps
    ms = min(ms_eager, ms_graph)
    line = {
        "metric": METRIC, "value": n_rays / (ms / 1e3) / 1e6, "unit": METRIC, "n_gpus": 1,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded clutter scene; rays generated on the GPU)",
        "config": {"workload": f"clutter-{a.objects}obj N{a.branching}L{a.leaf} {w}x{h} frame on the "
                               f"GPU: camera rays, primary, shadow + {spp} cosine AO rays per hit "
                               "generated from the hits, AO factor",
                   "rays_per_step": n_rays, "primary": n_prim, "shadow": n_sh, "ao": n_ao,
                   "ms_eager": ms_eager, "ms_graph": ms_graph, "graph_equals_eager": graph_ok,
                   "oracle_equal_on_20k_samples": checks, "setup_s": round(setup_s, 1),
                   "plan": "primary per-ray (local stacks); shadow persistent policy 2, refill 16; "
                           "AO persistent policy 2, refill 24, 6x10x10 direction bins, "
                           "child-index push order"},
        "e2e": {"value": n_rays / e2e_s / 1e6, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(w * h * 4)},
        "clocks": clocks,
        # camera rays, primary trace, secondary rays, shadow trace (+ queue clear
        # is a memset), four reorder passes + AO trace, AO factor
        "gpu_launches": 10 * a.steps,
    }
    print(json.dumps(line))


def run_sweep(a):
    """The 1M-triangle clutter frame for every N, L in {4, 8, 12, 16}^2:
    plain per-ray against ray-stream traversal, the persistent kernel and the
    default bench's per-batch plan, Mrays/s of the whole frame (primary +
    shadow + 8 AO per hit)."""
    import torch
    import bvhraytracer_gb300 as pkg
    dev = torch.device("cuda", 0)
    tris, bvh0, primary = make_frame(a)
    sc0 = pkg.Scene(bvh0)
    d_p = torch.from_numpy(primary).to(dev)
    prims = pkg.hit_prims(sc0.trace(d_p)["hits"].cpu().numpy())
    shadow, ao = secondaries(a, tris, primary, prims)
    batches = [(d_p, "closest"), (torch.from_numpy(shadow).to(dev), "any"),
               (torch.from_numpy(ao).to(dev), "any")]
    n_rays = sum(int(r.shape[0]) for r, _ in batches)
    stream = torch.cuda.current_stream(dev)
    table = {}
    for n in (4, 8, 12, 16):
        for l in (4, 8, 12, 16):
            bvh = pkg.Bvh(tris, n, l)
            sc = pkg.Scene(bvh)
            row = {}
            ref = None
            # "this_method": the default bench's usual plan per batch (primary
            # per-ray; shadow persistent policy 2; AO persistent policy 2,
            # refill 24, direction bins K = 10, child-index push order).
            plan = [{"scheme": "per_ray"}, {"scheme": "persistent", "policy": 2, "refill": 16},
                    {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10,
                     "any_order": True}]
            for name, o in (("per_ray", {"scheme": "per_ray"}),
                            ("stream_wg16", {"scheme": "stream"}),
                            ("persistent", {"scheme": "persistent", "policy": 2, "refill": 16}),
                            ("this_method", plan)):
                ms = 0.0
                outs = []
                try:
                    for bi, (r, k) in enumerate(batches):
                        ob = o[bi] if isinstance(o, list) else o
                        t, out = _time_trace(sc, r, k, ob, max(1, a.steps // 2), stream)
                        ms += t
                        outs.append(out["hits" if k == "closest" else "occluded"].view(torch.uint8))
                except pkg.BvhgpuError as e:
                    row[name] = {"unsupported": str(e)}
                    continue
                if ref is None:
                    ref = outs
                same = all(torch.equal(x, y) for x, y in zip(outs, ref))
                row[name] = {"ms": round(ms, 3), "mrays_per_s": round(n_rays / ms / 1e3, 1),
                             "equal_to_per_ray": bool(same)}
            sc.status()
            table[f"N{n}L{l}"] = row
            del sc, bvh
    best = max(table, key=lambda k: table[k]["this_method"]["mrays_per_s"])
    line = {
        "metric": METRIC, "value": table[best]["this_method"]["mrays_per_s"], "unit": METRIC,
        "n_gpus": 1, "steps": a.steps, "warmup": 1, "ms_per_step": table[best]["this_method"]["ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded clutter scene standing in for the reference's glTF scenes)",
        "config": {"workload": workload_name(a).replace(f"N{a.branching}L{a.leaf}", "N,L sweep"),
                   "rays_per_step": n_rays, "best": best, "by_nl": table},
    }
    print(json.dumps(line))


def run_aolaunch(a):
    """The frame's AO batch alone, an evenly strided sample of --ao-sample
    rays, traced with the bench's AO plan (persistent kernel, speculative
    any-hit policy 2, refill 24, 6 x 10 x 10 direction bins, child-index push
    order; or the --plan specs "scheme,policy,refill,reorder,any_order"
    joined by ';', each timed in turn and checked against the first)
    --warmup + --steps times; node format --nodes. Prints per plan the device
    time and the algorithmic bytes per launch. It is the case the ncu DRAM
    captures of the AO launch use (a launch of about 2M rays keeps a capture
    short); the bytes per ray they measure scale with the ray count."""
    import torch
    import bvhraytracer_gb300 as pkg
    dev = torch.device("cuda", 0)
    tris, bvh, primary = make_frame(a)
    plain = pkg.Scene(bvh)
    scene = (plain if a.nodes == "fp32" and a.top_levels == 0 else
             pkg.Scene(bvh, node_format=a.nodes, top_levels=a.top_levels))
    hits = plain.trace(torch.from_numpy(primary).to(dev))["hits"]
    _, ao = secondaries(a, tris, primary, pkg.hit_prims(hits.cpu().numpy()))
    idx = np.unique(np.linspace(0, ao.shape[0] - 1, min(a.ao_sample, ao.shape[0])).astype(np.int64))
    rays = torch.from_numpy(ao[idx]).to(dev)
    plans = [{"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10, "any_order": True}]
    if a.plan:
        plans = []
        for spec in a.plan.split(";"):
            f = spec.split(",")
            plans.append({"scheme": f[0], "policy": int(f[1]), "refill": int(f[2]),
                          "reorder": int(f[3]), "any_order": bool(int(f[4]))})
    c = scene.trace(rays, kind="any", counters=True, scheme="persistent", policy=0, refill=24)
    cs = c["counters"].to(torch.int64).sum(0).cpu().numpy()
    alg = int(cs[0]) * scene.node_record_bytes + int(cs[4]) * 36
    stream = torch.cuda.current_stream(dev)
    first = None
    for plan in plans:
        out = torch.empty(rays.shape[0], dtype=torch.uint8, device=dev)
        for _ in range(a.warmup):
            scene.trace(rays, kind="any", out=out, **plan)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            scene.trace(rays, kind="any", out=out, **plan)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / max(a.steps, 1)
        scene.status()
        if first is None:
            first = out.clone()
        print(json.dumps({
            "metric": METRIC, "value": rays.shape[0] / (ms / 1e3) / 1e6, "unit": METRIC,
            "ms_per_launch": ms, "rays": int(rays.shape[0]), "workload": workload_name(a),
            "nodes": a.nodes, "top_levels": a.top_levels, "plan": plan,
            "triangles": int(bvh.info["n_tris"]),
            "same_as_first_plan": bool(torch.equal(out, first)),
            "algorithmic_bytes_per_launch": alg, "node_record_bytes": scene.node_record_bytes,
            "node_visits_per_ray": float(cs[0]) / rays.shape[0],
            "tri_tests_per_ray": float(cs[4]) / rays.shape[0]}))


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "batch64":
        run_batch(a)
    elif a.workload == "adjoint":
        run_adjoint(a)
    elif a.workload == "scale8m":
        run_scale(a)
    elif a.workload == "terrain":
        run_terrain(a)
    elif a.workload == "sweep":
        run_sweep(a)
    elif a.workload == "gpuframe":
        run_gpuframe(a)
    elif a.workload == "aolaunch":
        run_aolaunch(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
