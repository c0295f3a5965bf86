"""Report files in the reference's formats, written from GPU counters and
timings, so its analysis scripts (Analysis/DataManager.py, which reads every
value as the first number after a fixed key) can consume GPU results.

* ``<name><problem>_Info.txt`` — CameraData::renderImage's traversal
  statistics (src/cameraData.h:241-325): per-ray node / leaf / box / triangle
  counts, success ratios, waste factors, traversal fullness and the per-depth
  node and leaf visit histograms, for primary and secondary rays, and the
  fullness sections (visits of nodes with x children and of leaves with x
  triangles per primary ray, with their averages) from the kernels'
  childFullness / primitiveFullness histograms.
* ``WorkGroupSize_<wg>_Version_<v>/...`` — CameraData::workGroupAnalysisPerImage
  (cameraData.h:660-1105): the primary / secondary whisker plots of the
  termination steps per workgroup, ``_WorkGroupData.txt`` (per step: average
  node and leaf work, unique nodes and leaves, accumulated terminations) and
  ``_WorkGroupUniqueWork.txt`` (per workgroup: node and leaf visits of its
  rays, unique nodes and leaves summed over its steps), from the stream
  kernel's step log (``Scene.trace(..., scheme="stream", counters=True,
  steps=S)``).
* ``<name><problem>_Perf.txt`` — CameraFast::renderImage's timing summary
  (src/cameraFast.h:147-161) with the device time of the frame. The GPU does
  not time rays and triangle tests separately, so those lines read ``n/a``
  (DataManager then records no value for them).
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np


@dataclass
class RayStats:
    """Sums over one ray batch: per-ray counters (``[n, 8]``: node visits,
    leaf visits, box tests, box hits, triangle tests, triangle hits, deepest
    stack, reserved) and the ``[2, 64]`` per-depth node / leaf visit
    histogram, as returned by ``Scene.trace(..., counters=True,
    depth_hist=True)``."""
    rays: int
    node_visits: int
    leaf_visits: int
    box_tests: int
    box_hits: int
    tri_tests: int
    tri_hits: int
    node_depth: np.ndarray
    leaf_depth: np.ndarray
    # visits of nodes with c children / leaves with c triangles ([17] each)
    child_fullness: np.ndarray | None = None
    prim_fullness: np.ndarray | None = None

    @classmethod
    def from_trace(cls, counters, depth_hist, rays_counted: int | None = None,
                   fullness=None) -> "RayStats":
        c = np.asarray(_host(counters), np.int64).reshape(-1, 8)
        h = np.asarray(_host(depth_hist), np.int64).reshape(2, -1)
        s = c.sum(0)
        f = None if fullness is None else np.asarray(_host(fullness), np.uint64).reshape(2, -1)
        return cls(int(rays_counted if rays_counted is not None else c.shape[0]), int(s[0]),
                   int(s[1]), int(s[2]), int(s[3]), int(s[4]), int(s[5]), h[0], h[1],
                   None if f is None else f[0], None if f is None else f[1])


def _host(x):
    if hasattr(x, "cpu"):
        return x.cpu().numpy()
    return x


def _fmt(v: float) -> str:
    # std::ostream's default float formatting: 6 significant digits.
    return f"{v:.6g}"


def _section(prefix: str, s: RayStats, branching: int) -> list[str]:
    f = 1.0 / max(s.rays, 1)
    waste = (s.leaf_visits + s.node_visits - s.rays) / float(max(s.node_visits * branching, 1))
    return [
        f"{prefix} intersections node: {_fmt(s.node_visits * f)}",
        f"{prefix} aabb intersections: {_fmt(s.box_tests * f)}",
        f"{prefix} aabb success ration: {_fmt(s.box_hits / max(s.box_tests, 1))}",
        f"{prefix} waste factor: {_fmt(1 - waste)}",
        f"{prefix} intersections leaf: {_fmt(s.leaf_visits * f)}",
        f"{prefix} primitive intersections: {_fmt(s.tri_tests * f)}",
        f"{prefix} primitive success ratio: {_fmt(s.tri_hits / max(s.tri_tests, 1))}",
    ]


def _fullness(title: str, avg: str, hist, bins: int, rays: int) -> list[str]:
    """One fullness section as CameraData writes it (cameraData.h:267-294):
    the float average sum(i * h[i]) / sum(h) (std::to_string) and per count
    h[i] / rays in float (bins = N + 1 or L + 1 entries)."""
    h = np.asarray(hist, np.uint64)[:bins]
    acc = np.float32(0)
    for i in range(bins):
        acc = np.float32(acc + np.float32(int(h[i]) * i))
    total = int(h.sum())
    acc = np.float32(acc / np.float32(total)) if total else np.float32("nan")
    factor = np.float32(1) / np.float32(max(rays, 1))
    out = [title, f"{avg}{float(acc):.6f}"]
    out += [f"{i} : {_fmt(float(np.float32(np.float32(int(h[i])) * factor)))}" for i in range(bins)]
    return out


def write_info(path: str, name: str, problem: str, branching: int, leaf_size: int,
               primary: RayStats, secondary: RayStats) -> str:
    """Writes ``<path>/<name><problem>_Info.txt``; returns the file name."""
    lines = [f"scenario {name} with branching factor of {branching} and leafsize of {leaf_size}",
             "intersections counts are normalized per Ray", ""]
    lines += _section("primary", primary, branching) + [""]
    lines += _section("secondary", secondary, branching) + [""]
    # Fullness is collected from primary rays only (collectPrimaryRayData,
    # cameraData.h:577-621).
    if primary.child_fullness is not None:
        lines += _fullness("intersections with nodes with x children :",
                           "average child fullness: ", primary.child_fullness, branching + 1,
                           primary.rays)
        lines += [""]
        lines += _fullness("intersections with leaf nodes with x primitives :",
                           "average leaf fullness: ", primary.prim_fullness, leaf_size + 1,
                           primary.rays)
    else:  # averages only, from the counters
        lines += ["intersections with nodes with x children :",
                  "average child fullness: "
                  f"{primary.box_tests / max(primary.node_visits, 1):.6f}", "",
                  "intersections with leaf nodes with x primitives :",
                  "average leaf fullness: "
                  f"{primary.tri_tests / max(primary.leaf_visits, 1):.6f}"]
    for title, hist, s in (("primary node intersections at depth x :", primary.node_depth, primary),
                           ("primary leaf intersections at depth x :", primary.leaf_depth, primary),
                           ("secondary node intersections at depth x :", secondary.node_depth,
                            secondary),
                           ("secondary leaf intersections at depth x :", secondary.leaf_depth,
                            secondary)):
        last = int(np.max(np.nonzero(hist)[0])) + 1 if np.any(hist) else 0
        lines += ["", title] + [f"{i} : {_fmt(hist[i] / max(s.rays, 1))}" for i in range(last)]
    os.makedirs(path, exist_ok=True)
    fn = os.path.join(path, f"{name}{problem}_Info.txt")
    with open(fn, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return fn


def write_perf(path: str, name: str, problem: str, branching: int, leaf_size: int, gang: int,
               node_memory: int, leaf_memory: int, total_seconds: float,
               average_depth: float, triangles: int) -> str:
    """Writes ``<path>/<name><problem>_Perf.txt``; returns the file name."""
    lines = [
        f"scenario {name} with branching factor of {branching} and leafsize of {leaf_size}",
        f"with a gang size of {gang}, a node meory of {node_memory}, and a leaf memory of "
        f"{leaf_memory}",
        f"Raytracer total time: {_fmt(total_seconds)}",
        "Time for all rays (SUM): n/a",
        "Time for triangle intersections (SUM): n/a",
        "Time all rays(sum) - triangle(sum): n/a",
        f"Average BVH depth: {_fmt(average_depth)}",
        f"Triangle Count: {triangles}",
    ]
    os.makedirs(path, exist_ok=True)
    fn = os.path.join(path, f"{name}{problem}_Perf.txt")
    with open(fn, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return fn


def average_leaf_depth(leaf_depth_hist_of_tree) -> float:
    """Mean depth over a histogram of leaves per depth."""
    h = np.asarray(leaf_depth_hist_of_tree, np.float64)
    return float((h * np.arange(h.shape[0])).sum() / max(h.sum(), 1.0))


def termination_steps(counters) -> np.ndarray:
    """Step at which each ray of a ray-stream traversal terminates, in the
    numbering of intersectWideAlternative's terminationsPerStep
    (compactNode.cpp:418-590): an inactive ray terminates at step 0, an
    active one after one node or leaf visit per step, i.e. at step
    node visits + leaf visits. The same counts hold for every scheme (the
    kernels visit the same nodes and leaves per ray)."""
    c = np.asarray(_host(counters), np.int64).reshape(-1, 8)
    return c[:, 0] + c[:, 1]


def _whisker_rows(steps: np.ndarray, group: int):
    """Per workgroup (median, min, max, average, standard deviation) of the
    termination steps, sorted by (median, max) like
    CameraData::workGroupAnalysisPerImage (cameraData.h:671-778)."""
    n = steps.shape[0] // group
    rows = []
    for i in range(n):
        d = np.sort(steps[i * group:(i + 1) * group])
        avg = float(np.float32(d.sum()) / np.float32(group))
        sd = float(np.sqrt(np.mean((d - avg) ** 2)))
        rows.append((int(d[int(group * 0.5)]), int(d[0]), int(d[-1]), avg, sd))
    rows.sort(key=lambda r: (r[0], r[2]))
    return rows


def termination_steps_from_log(step_stats, step_count, n_groups: int) -> np.ndarray:
    """Termination step of every ray of the first ``n_groups`` packets from
    the stream kernel's step log: step s repeated terminations[s] times per
    packet, as workGroupAnalysisPerImage expands terminationsPerStep
    (cameraData.h:727-741). Valid for either wide schedule."""
    st = np.asarray(_host(step_stats), np.int64)
    ct = np.asarray(_host(step_count), np.int64)
    out = []
    for i in range(n_groups):
        k = int(ct[i])
        if k > st.shape[1]:
            raise ValueError("step log shorter than a workgroup's traversal: trace with more steps")
        out.append(np.repeat(np.arange(k), st[i, :k, 4]))
    return np.concatenate(out) if out else np.zeros(0, np.int64)


def write_workgroup_whisker(path: str, name: str, problem: str, camera_name: str,
                            workgroup: int, wide_alternative: int, primary, secondary,
                            n_groups: int = 0) -> list[str]:
    """Writes ``WorkGroupSize_<wg>_Version_<v>/<name><problem><camera>_
    {Primary,Secondary}WorkGroupWiskerPlot.txt``. ``primary`` / ``secondary``:
    per-ray counters of rays in workgroup order (workgroup^2 consecutive rays
    per workgroup, one secondary ray per pixel; a ray terminates at step node
    visits + leaf visits, the intersectWideAlternative schedule), or a
    ``(step_stats, step_count)`` step log of either schedule with the number
    of workgroups ``n_groups``."""
    folder = os.path.join(path, f"WorkGroupSize_{workgroup}_Version_{wide_alternative}")
    os.makedirs(folder, exist_ok=True)
    out = []
    for kind, c in (("Primary", primary), ("Secondary", secondary)):
        steps = (termination_steps_from_log(c[0], c[1], n_groups) if isinstance(c, tuple)
                 else termination_steps(c))
        rows = _whisker_rows(steps, workgroup * workgroup)
        fn = os.path.join(folder, f"{name}{problem}{camera_name}_{kind}WorkGroupWiskerPlot.txt")
        with open(fn, "w") as fh:
            fh.write("median, min, max, lowerStdDeviation, upperStdDeviation\n")
            for r in rows:
                fh.write(f"{r[0]}, {r[1]}, {r[2]}, {_fmt(r[3])}, {_fmt(r[4])}\n")
        out.append(fn)
    return out


def _f32(x) -> np.float32:
    return np.float32(x)


def write_workgroup_data(path: str, name: str, problem: str, camera_name: str, workgroup: int,
                         wide_alternative: int, n_groups: int, primary_steps, primary_step_count,
                         secondary_steps, secondary_step_count, primary_counters,
                         secondary_counters) -> list[str]:
    """Writes ``WorkGroupSize_<wg>_Version_<v>/<name><problem><camera>_
    WorkGroupData.txt`` and ``..._WorkGroupUniqueWork.txt`` like
    CameraData::workGroupAnalysisPerImage (cameraData.h:809-1105), from the
    step logs of ``Scene.trace(..., scheme="stream", counters=True,
    steps=S)`` (``[packets, S, 5]`` and ``[packets]``) and the per-ray
    counters, for the first ``n_groups`` packets (the reference's
    (width / workGroupSize) * (height / workGroupSize) full workgroups, which
    come first when the width is a multiple of the workgroup size).

    The reference's quirks are kept: the step range is the longest primary
    log (its second size check reads the primary log again), averages are
    float sums in workgroup order, unique-count averages run over workgroups
    that touched at least one node (leaf), terminations are averaged over
    all workgroups and accumulated over steps."""
    wsq = workgroup * workgroup

    def logs(steps, count):
        st = np.asarray(_host(steps), np.int64)
        ct = np.asarray(_host(count), np.int64)
        if np.any(ct[:n_groups] > st.shape[1]):
            raise ValueError("step log shorter than a workgroup's traversal: trace with more steps")
        return st[:n_groups], ct[:n_groups]

    ps, pc = logs(primary_steps, primary_step_count)
    ss, scnt = logs(secondary_steps, secondary_step_count)
    max_size = int(pc.max()) if n_groups else 0
    folder = os.path.join(path, f"WorkGroupSize_{workgroup}_Version_{wide_alternative}")
    os.makedirs(folder, exist_ok=True)
    header = ("stepId, avgPrimaryNodeWork, avgPrimaryNodeUnique, avgPrimaryLeafWork, "
              "avgPrimaryLeafUnique, avgPrimaryRayTermination, primaryNodeWorkMax, "
              "primaryNodeWorkMin, primaryLeafWorkMax, primaryLeafWorkMin, avgSecondaryNodeWork, "
              "avgSecondaryNodeUnique, avgSecondaryLeafWork, avgSecondaryLeafUnique, "
              "avgSecondaryRayTermination, secondaryNodeWorkMax, secondaryNodeWorkMin, "
              "secondaryLeafWorkMax, secondaryLeafWorkMin")
    lines = [header]
    term_prev = [_f32(0), _f32(0)]
    groups = _f32(n_groups)
    for j in range(max_size):
        row = [str(j)]
        for side, (st, ct) in enumerate(((ps, pc), (ss, scnt))):
            nw = lw = un = ul = tr = _f32(0)
            cnt = ucn = ucl = 0
            umax_n = umax_l = 0
            umin_n = umin_l = wsq + 1
            for i in range(n_groups):
                if ct[i] <= j:
                    continue
                cnt += 1
                rec = st[i, j]
                nw = _f32(nw + _f32(rec[0]))
                lw = _f32(lw + _f32(rec[2]))
                un = _f32(un + _f32(rec[1]))
                ul = _f32(ul + _f32(rec[3]))
                tr = _f32(tr + _f32(rec[4]))
                if rec[1] != 0:
                    ucn += 1
                    umax_n, umin_n = max(int(rec[1]), umax_n), min(int(rec[1]), umin_n)
                if rec[3] != 0:
                    ucl += 1
                    umax_l, umin_l = max(int(rec[3]), umax_l), min(int(rec[3]), umin_l)
            cnt, ucn, ucl = max(cnt, 1), max(ucn, 1), max(ucl, 1)
            umin_n = 0 if umin_n == wsq + 1 else umin_n
            umin_l = 0 if umin_l == wsq + 1 else umin_l
            tr = _f32(tr / groups)
            if j != 0:
                tr = _f32(tr + term_prev[side])
            term_prev[side] = tr
            row += [_fmt(float(_f32(nw / _f32(cnt)))), _fmt(float(_f32(un / _f32(ucn)))),
                    _fmt(float(_f32(lw / _f32(cnt)))), _fmt(float(_f32(ul / _f32(ucl)))),
                    _fmt(float(tr)), str(umax_n), str(umin_n), str(umax_l), str(umin_l)]
        lines.append(", ".join(row))
    fn_data = os.path.join(folder, f"{name}{problem}{camera_name}_WorkGroupData.txt")
    with open(fn_data, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    # Per workgroup: node / leaf visits summed over its rays (with their max
    # and min) and the unique nodes / leaves summed over its steps.
    pcn = np.asarray(_host(primary_counters), np.int64).reshape(-1, 8)
    scn = np.asarray(_host(secondary_counters), np.int64).reshape(-1, 8)
    lines = ["loadedPrimaryNodes, loadedPrimaryLeafs, loadedPrimaryNodesMax, loadedPrimaryLeafsMax, "
             "loadedPrimaryNodesMin, loadedPrimaryLeafsMin, loadedSecondaryNodes, "
             "loadedSecondaryLeafs, loadedSecondaryNodesMax, loadedSecondaryLeafsMax, "
             "loadedSecondaryNodesMin, loadedSecondaryLeafsMin, loadedWidePrimaryNodes, "
             "loadedWidePrimaryLeafs, loadedWideSecondaryNodes, loadedWideSecondaryLeafs"]
    for i in range(n_groups):
        row = []
        for c in (pcn, scn):
            g = c[i * wsq:(i + 1) * wsq]
            nodes = leaves = _f32(0)
            for k in range(g.shape[0]):
                nodes = _f32(nodes + _f32(g[k, 0]))
                leaves = _f32(leaves + _f32(g[k, 1]))
            # minima start at 1000 and read 0 when no ray went below it
            mn = [int(g[:, a].min(initial=1000)) for a in (0, 1)]
            mn = [0 if m == 1000 else m for m in mn]
            row += [_fmt(float(nodes)), _fmt(float(leaves)), str(int(g[:, 0].max(initial=0))),
                    str(int(g[:, 1].max(initial=0))), str(mn[0]), str(mn[1])]
        for st, ct in ((ps, pc), (ss, scnt)):
            k = int(ct[i])
            row += [_fmt(float(int(st[i, :k, 1].sum()))), _fmt(float(int(st[i, :k, 3].sum())))]
        lines.append(", ".join(row))
    fn_unique = os.path.join(folder, f"{name}{problem}{camera_name}_WorkGroupUniqueWork.txt")
    with open(fn_unique, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return [fn_data, fn_unique]
