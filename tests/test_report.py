"""Report files in the reference's formats: every value the reference's
analysis script reads (the first number after its key) is present and
equals the statistic computed from the counters."""
import numpy as np
import pytest

from bvhraytracer_gb300 import report as R


def first_number(text: str, key: str):
    """DataManager.gatherVariable: first token after the key that parses as
    a float, on the line containing the key (Analysis/DataManager.py:397-407)."""
    hits = [ln for ln in text.splitlines() if key in ln]
    assert len(hits) == 1, key
    for t in hits[0].split():
        try:
            return float(t)
        except ValueError:
            pass
    return None


def _stats(seed, n):
    rng = np.random.default_rng(seed)
    c = rng.integers(0, 50, (n, 8))
    h = np.zeros((2, 64), np.int64)
    h[0, :5] = rng.integers(0, 100, 5)
    h[1, 2:6] = rng.integers(0, 100, 4)
    return R.RayStats.from_trace(c, h), c, h


def test_info_file_values(tmp_path):
    p, cp, hp = _stats(0, 100)
    s, cs, _ = _stats(1, 300)
    fn = R.write_info(str(tmp_path), "clutter", "_b8_l8", 8, 8, p, s)
    text = open(fn).read()
    assert first_number(text, "primary intersections node:") == float(f"{cp[:, 0].sum() / 100:.6g}")
    assert first_number(text, "secondary intersections leaf:") == float(f"{cs[:, 1].sum() / 300:.6g}")
    ratio = cp[:, 3].sum() / cp[:, 2].sum()
    assert abs(first_number(text, "primary aabb success ration:") - ratio) < 1e-5
    waste = 1 - (cp[:, 1].sum() + cp[:, 0].sum() - 100) / (cp[:, 0].sum() * 8)
    assert abs(first_number(text, "primary waste factor:") - waste) < 1e-5
    assert abs(first_number(text, "average child fullness:") - cp[:, 2].sum() / cp[:, 0].sum()) < 1e-5
    assert "primary node intersections at depth x :" in text
    assert f"4 : {hp[0, 4] / 100:.6g}" in text


def test_perf_file_values(tmp_path):
    fn = R.write_perf(str(tmp_path), "clutter", "_b8_l8_mb8_ml8", 8, 8, 4, 8, 8, 0.00958, 14.2,
                      999744)
    text = open(fn).read()
    assert first_number(text, "Raytracer total time:") == 0.00958
    assert first_number(text, "Time for triangle intersections (SUM):") is None
    assert first_number(text, "Triangle Count:") == 999744


def test_termination_steps_match_stream_oracle():
    """The termination step of every ray (node + leaf visits) reproduces the
    per-step termination counts of the stream traversal."""
    from oracle import oracle as O
    from tests import _scenes as TS
    tris, b, cv = TS.bvh("clutter120", 8, 8)
    rays = TS.clutter_rays(tris)[:256 * 4]
    rays[5, 0] = np.nan
    r = O.trace_instrumented(cv, rays, False, packet=256)
    steps = R.termination_steps(r["counters"])
    assert steps[5] == 0 and (steps[np.arange(len(steps)) != 5] > 0).all()
    assert np.array_equal(steps, r["counters"][:, 0].astype(np.int64) + r["counters"][:, 1])


def test_whisker_file(tmp_path):
    c = np.zeros((8, 8), np.int64)
    c[:, 0] = [3, 1, 2, 5, 9, 9, 9, 9]
    c[:, 1] = [1, 1, 1, 1, 0, 1, 2, 3]
    files = R.write_workgroup_whisker(str(tmp_path), "s", "_b8_l8", "_c0", 2, 1, c, c)
    lines = open(files[0]).read().splitlines()
    assert lines[0] == "median, min, max, lowerStdDeviation, upperStdDeviation"
    # groups: [4,2,3,6] -> median 4 (index 2 of sorted 2,3,4,6), [9,10,11,12] -> 11
    assert lines[1].startswith("4, 2, 6, 3.75") and lines[2].startswith("11, 9, 12, 10.5")


def test_workgroup_data_files(tmp_path):
    """_WorkGroupData.txt / _WorkGroupUniqueWork.txt from step logs of two
    2x2 workgroups, against values worked out by hand from
    cameraData.h:809-1105 (averages over active workgroups, unique averages
    over workgroups that touched a node / leaf, terminations averaged over
    all workgroups and accumulated, step range of the primary logs)."""
    from bvhraytracer_gb300 import report as R
    P = np.zeros((2, 4, 5), np.int32)
    P[0, :3] = [[4, 1, 0, 0, 0], [4, 2, 0, 0, 1], [3, 1, 0, 0, 3]]
    P[1, :2] = [[4, 1, 0, 0, 0], [0, 0, 4, 3, 4]]
    S = np.zeros((2, 4, 5), np.int32)
    S[0, :2] = [[2, 1, 0, 0, 2], [2, 1, 0, 0, 2]]
    S[1, :4] = [[4, 1, 0, 0, 0], [4, 2, 0, 0, 0], [0, 0, 4, 2, 2], [2, 1, 0, 0, 2]]
    pc = np.zeros((8, 8), np.int32)
    pc[:, 0] = [3, 2, 2, 1, 1, 1, 1, 1]
    pc[:, 1] = [0, 1, 0, 2, 1, 1, 1, 1]
    sc = np.zeros((8, 8), np.int32)
    sc[:, 0] = [2, 2, 0, 0, 3, 2, 1, 2]
    sc[:, 1] = [0, 0, 0, 0, 1, 1, 0, 0]
    data, unique = R.write_workgroup_data(str(tmp_path), "scene", "_p", "_cam", 2, 1, 2, P,
                                          np.array([3, 2]), S, np.array([2, 4]), pc, sc)
    assert data.endswith("WorkGroupSize_2_Version_1/scene_p_cam_WorkGroupData.txt")
    lines = open(data).read().splitlines()
    assert lines[0].startswith("stepId, avgPrimaryNodeWork, avgPrimaryNodeUnique")
    assert lines[1:] == ["0, 4, 1, 0, 0, 0, 1, 1, 0, 0, 3, 1, 0, 0, 1, 1, 1, 0, 0",
                         "1, 2, 2, 2, 3, 2.5, 2, 2, 3, 3, 3, 1.5, 0, 0, 2, 2, 1, 0, 0",
                         "2, 3, 1, 0, 0, 4, 1, 1, 0, 0, 0, 0, 4, 2, 3, 0, 0, 2, 2"]
    lines = open(unique).read().splitlines()
    assert lines[0].startswith("loadedPrimaryNodes, loadedPrimaryLeafs")
    assert lines[1:] == ["8, 3, 3, 2, 1, 0, 4, 0, 2, 0, 0, 0, 4, 0, 2, 0",
                         "4, 4, 1, 1, 1, 1, 8, 2, 3, 1, 1, 0, 1, 3, 4, 2"]
    with pytest.raises(ValueError):
        R.write_workgroup_data(str(tmp_path), "s", "", "", 2, 1, 2, P, np.array([5, 2]), S,
                               np.array([2, 4]), pc, sc)


def test_whisker_from_step_log_matches_counters():
    """Termination steps expanded from a step log equal node + leaf visits
    per ray for the alternative schedule (here a synthetic log built from
    per-ray visit counts of two 2x2 workgroups)."""
    from bvhraytracer_gb300 import report as R
    visits = np.array([[3, 1], [2, 0], [0, 0], [4, 2], [1, 1], [2, 2], [5, 0], [3, 3]])
    c = np.zeros((8, 8), np.int32)
    c[:, 0], c[:, 1] = visits[:, 0], visits[:, 1]
    steps = c[:, 0] + c[:, 1]
    log = np.zeros((2, 12, 5), np.int32)
    count = np.zeros(2, np.int32)
    for g in range(2):
        s = steps[g * 4:(g + 1) * 4]
        count[g] = s.max() + 1
        for v in s:
            log[g, v, 4] += 1
    from_log = R.termination_steps_from_log(log, count, 2)
    want = np.concatenate([np.sort(steps[:4]), np.sort(steps[4:])])
    assert np.array_equal(from_log, want)
    assert R._whisker_rows(from_log, 4) == R._whisker_rows(steps, 4)


def test_info_file_fullness_sections(tmp_path):
    """The per-count fullness lines of CameraData (cameraData.h:267-294):
    visits of nodes with x children and of leaves with x triangles per
    primary ray, and their float averages, from the kernels' histograms."""
    p, _, _ = _stats(0, 100)
    s, _, _ = _stats(1, 300)
    full = np.zeros((2, 17), np.uint64)
    full[0, 2], full[0, 4] = 3, 5
    full[1, 1], full[1, 3] = 7, 1
    p = R.RayStats.from_trace(np.zeros((100, 8)), np.zeros((2, 64)), fullness=full)
    fn = R.write_info(str(tmp_path), "clutter", "_b4_l3", 4, 3, p, s)
    lines = open(fn).read().splitlines()
    i = lines.index("intersections with nodes with x children :")
    assert lines[i + 1] == "average child fullness: 3.250000"
    assert lines[i + 2:i + 7] == ["0 : 0", "1 : 0", "2 : 0.03", "3 : 0", "4 : 0.05"]
    j = lines.index("intersections with leaf nodes with x primitives :")
    assert lines[j + 1] == "average leaf fullness: 1.250000"
    assert lines[j + 2:j + 6] == ["0 : 0", "1 : 0.07", "2 : 0", "3 : 0.01"]
    assert first_number("\n".join(lines), "average leaf fullness:") == 1.25
