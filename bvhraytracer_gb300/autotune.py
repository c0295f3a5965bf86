"""Autotuner: picks, per scene and per ray batch, the traversal configuration
with the lowest measured time.

Candidates cover the knobs the reference exposes in config.txt (branching
factor N and leaf size L: a scene is built per (N, L) pair) plus the GPU
ones: traversal scheme (per-ray, ray-stream with its workgroup size,
persistent with its refill threshold and divergence policy), stack placement
(shared or local memory), whether the rays are grouped by direction first
(reorder), node format (FP32 / Q8) and how many top levels are staged in
shared memory. Every
candidate gives the same hits (the kernels are bit-exact with one another and
Q8 keeps hit sets identical), so the choice only changes speed.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

from . import Bvh, Scene

DEFAULT_OPTIONS = (
    {"scheme": "per_ray", "block": 128},
    {"scheme": "per_ray", "block": 64},
    {"scheme": "per_ray", "block": 128, "stack": "local"},
    {"scheme": "stream", "workgroup": 8},
    {"scheme": "stream", "workgroup": 16},
    {"scheme": "persistent", "policy": 0, "refill": 8},
    {"scheme": "persistent", "policy": 0, "refill": 16},
    {"scheme": "persistent", "policy": 1, "refill": 8},
    {"scheme": "persistent", "policy": 2, "refill": 8},
    {"scheme": "persistent", "policy": 2, "refill": 16},
    {"scheme": "per_ray", "block": 128, "reorder": 8},
    {"scheme": "persistent", "policy": 0, "refill": 16, "reorder": 8},
    {"scheme": "persistent", "policy": 2, "refill": 16, "reorder": 8},
    {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 8},
    {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10},
    # any-hit batches only: child-index push order
    {"scheme": "persistent", "policy": 2, "refill": 24, "reorder": 10, "any_order": True},
    {"scheme": "persistent", "policy": 2, "refill": 16, "any_order": True},
    # any-hit batches only: two leaves set aside per lane, tested per lane / warp-wide
    {"scheme": "persistent", "policy": 3, "refill": 16, "reorder": 10, "any_order": True},
    {"scheme": "persistent", "policy": 4, "refill": 24, "reorder": 10, "any_order": True},
)
DEFAULT_LAYOUTS = (("fp32", 0), ("fp32", 2), ("q8", 2))


@dataclass
class Plan:
    """Best configuration per batch: (layout, trace options, ms)."""
    choices: list = field(default_factory=list)
    table: dict = field(default_factory=dict)

    def describe(self) -> list:
        return [{"layout": f"{fmt}/top{top}", **opts, "ms": round(ms, 4)}
                for (fmt, top), opts, ms in self.choices]


def _time(scene, rays, kind, opts, profile, reps):
    import torch
    st = torch.cuda.current_stream(rays.device)
    scene.trace(rays, kind=kind, profile=profile, **opts)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        scene.trace(rays, kind=kind, profile=profile, **opts)
    e1.record(st)
    torch.cuda.synchronize(rays.device)
    return e0.elapsed_time(e1) / reps


def one_layout(table: dict, n_batches: int, mixed_ms: float, margin: float = 0.03):
    """The layout to trace every batch of a plan with, or None to keep the
    per-batch layouts. ``table`` maps (batch, layout, options) to ms. Batches
    in different layouts go through different scenes, so the host-buffer
    entry points run one pipeline (and one synchronisation) per scene; one
    layout for all batches is kept unless the mixed plan is faster by more
    than ``margin`` of its time."""
    per_layout = {}
    for (bi, lay, _), ms in table.items():
        best = per_layout.setdefault(lay, [None] * n_batches)
        if best[bi] is None or ms < best[bi]:
            best[bi] = ms
    totals = {lay: sum(b) for lay, b in per_layout.items() if all(x is not None for x in b)}
    if not totals:
        return None
    lay = min(totals, key=totals.get)
    return lay if totals[lay] <= mixed_ms * (1.0 + margin) else None


def tune_scene(bvh: Bvh, batches, *, profile: str = "instrumented", layouts=DEFAULT_LAYOUTS,
               options=DEFAULT_OPTIONS, reps: int = 3, device: int = 0, scenes=None,
               layout_margin: float = 0.03):
    """Times every (layout, options) candidate on each ``(rays, kind)`` batch
    (device tensors) and returns (plan, scenes by layout). All batches share
    one layout unless mixing layouts saves more than ``layout_margin`` of the
    time (see one_layout)."""
    scenes = dict(scenes or {})
    plan = Plan()
    for fmt, top in layouts:
        if (fmt, top) not in scenes:
            scenes[(fmt, top)] = Scene(bvh, node_format=fmt, top_levels=top, device=device)
    for bi, (rays, kind) in enumerate(batches):
        best = None
        for (lay, sc), opts in itertools.product(scenes.items(), options):
            if lay[0] != "fp32" and opts["scheme"] == "stream":
                continue
            if (opts.get("any_order") or opts.get("policy", 0) >= 3) and kind != "any":
                continue
            ms = _time(sc, rays, kind, opts, profile, reps)
            plan.table[(bi, lay, tuple(sorted(opts.items())))] = ms
            if best is None or ms < best[2]:
                best = (lay, opts, ms)
        plan.choices.append(best)
    lay = one_layout(plan.table, len(batches), sum(c[2] for c in plan.choices), layout_margin)
    if lay is not None:
        for bi, c in enumerate(plan.choices):
            if c[0] == lay:
                continue
            key = min((k for k in plan.table if k[0] == bi and k[1] == lay), key=plan.table.get)
            plan.choices[bi] = (lay, dict(key[2]), plan.table[key])
    return plan, scenes


def tune_branching(tris, batches_fn, *, pairs=((4, 4), (4, 8), (8, 4), (8, 8), (16, 4), (16, 8),
                                              (16, 16)),
                   profile: str = "instrumented", reps: int = 2, device: int = 0,
                   time_fn=None, prefer=None, margin: float = 0.0, **kw):
    """Also picks N and L: builds a BVH per pair, tunes each, returns the pair
    with the lowest total time. ``batches_fn(scene)`` returns the batches to
    time for a scene (secondary rays may depend on the primary hits).
    ``time_fn(scene, batches)``, when given, times the call the batches will
    actually run in (for instance the multi-scene launch of bvhgpu_trace_jobs)
    and returns its milliseconds; the plan then records that call.
    ``prefer`` (a pair among ``pairs``) is kept unless the fastest pair beats
    it by more than the fraction ``margin``: timings of short launches are
    noisy, and a pair shared by many scenes keeps their jobs in one launch
    group."""
    best = None
    kept = None
    results = {}
    for n, l in pairs:
        bvh = Bvh(tris, n, l)
        scene = Scene(bvh, device=device)
        batches = batches_fn(scene)
        if time_fn is not None:
            ms = float(time_fn(scene, batches))
            plan = Plan(choices=[(("fp32", 0), {"scheme": "time_fn"}, ms)])
            scenes = {("fp32", 0): scene}
        else:
            plan, scenes = tune_scene(bvh, batches, profile=profile, reps=reps, device=device,
                                      scenes={("fp32", 0): scene}, **kw)
        total = sum(ms for _, _, ms in plan.choices)
        results[(n, l)] = total
        if (n, l) == prefer:
            kept = (total, (n, l), bvh, plan, scenes)
        if best is None or total < best[0]:
            best = (total, (n, l), bvh, plan, scenes)
    if kept is not None and best[0] >= kept[0] * (1.0 - margin):
        best = kept
    return best, results
