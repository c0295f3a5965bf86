"""C ABI: the library loads, exports every declared entry point, and rejects
bad arguments with status codes (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import bvhraytracer_gb300 as pkg
from bvhraytracer_gb300 import _native as N

HEADER = Path(__file__).resolve().parent.parent / "include" / "bvhgpu.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\s*\*)\s+(bvhgpu_\w+)\s*\(", text, re.M)))


def test_header_declares_functions():
    names = declared_functions()
    assert len(names) >= 14
    assert "bvhgpu_trace" in names and "bvhgpu_bvh_build" in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(N.LIB_PATH))
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in bvhgpu.h but not exported"


def test_python_binding_covers_header():
    assert set(declared_functions()) == set(N.EXPORTED)


def test_status_codes_match_header():
    text = HEADER.read_text()
    codes = dict(re.findall(r"#define (BVHGPU_(?:OK|ERR_\w+))\s+(\d+)", text))
    assert int(codes["BVHGPU_OK"]) == N.OK
    assert int(codes["BVHGPU_ERR_BAD_ARG"]) == N.ERR_BAD_ARG
    assert int(codes["BVHGPU_ERR_STACK_OVERFLOW"]) == N.ERR_STACK_OVERFLOW
    assert int(codes["BVHGPU_ERR_UNSUPPORTED"]) == N.ERR_UNSUPPORTED
    assert int(codes["BVHGPU_ERR_NO_DEVICE"]) == N.ERR_NO_DEVICE


def test_struct_sizes_match_header_layout():
    assert C.sizeof(N.BuildParams) == 24
    assert C.sizeof(N.SceneParams) == 20
    assert C.sizeof(N.TraceOpts) == 52
    assert C.sizeof(N.Job) == 56


def _tri():
    return np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)


@pytest.mark.parametrize("n,l", [(1, 4), (17, 4), (4, 0), (4, 17)])
def test_build_rejects_bad_sizes(n, l):
    with pytest.raises(pkg.BvhgpuError) as e:
        pkg.Bvh(_tri(), n, l, sah=1.0)
    assert e.value.code == N.ERR_BAD_ARG


def test_build_rejects_null_and_empty():
    lib = N.lib()
    p = N.BuildParams(4, 4, 1, 1, 1.0, 1)
    h = C.c_void_p()
    assert lib.bvhgpu_bvh_build(None, 1, C.byref(p), C.byref(h)) == N.ERR_BAD_ARG
    t = _tri()
    assert lib.bvhgpu_bvh_build(t.ctypes.data, 0, C.byref(p), C.byref(h)) == N.ERR_BAD_ARG
    assert lib.bvhgpu_bvh_build(t.ctypes.data, 1, None, C.byref(h)) == N.ERR_BAD_ARG
    assert b"null" in lib.bvhgpu_last_error()


def test_build_rejects_non_finite_and_degenerate_only():
    t = _tri().copy()
    t[0, 4] = np.nan
    with pytest.raises(pkg.BvhgpuError):
        pkg.Bvh(t, 4, 4)
    deg = np.zeros((3, 9), np.float32)  # all zero-area
    with pytest.raises(pkg.BvhgpuError):
        pkg.Bvh(deg, 4, 4)


def test_build_rejects_unsorted_splits():
    with pytest.raises(pkg.BvhgpuError) as e:
        pkg.Bvh(_tri(), 4, 4, sort_each_split=False)
    assert e.value.code == N.ERR_UNSUPPORTED


def test_trace_rejects_null_scene_and_options():
    lib = N.lib()
    o = N.TraceOpts(0, 0, 0, 16, 128, 0, 0, 0, 0, 0, 0)
    assert lib.bvhgpu_trace(None, None, 1, C.byref(o), None, None, None, None, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_trace_host(None, None, 1, C.byref(o), None, None, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_scene_status(None, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_scene_free(None) == N.OK


def test_scene_create_without_device_reports_no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    b = pkg.Bvh(_tri(), 4, 4)
    with pytest.raises(pkg.BvhgpuError) as e:
        pkg.Scene(b)
    assert e.value.code == N.ERR_NO_DEVICE


def _stof(text: str) -> float:
    """Decimal text rounded straight to the nearest float32 (std::stof)."""
    from fractions import Fraction
    x = Fraction(text)
    c = np.float32(float(text))
    cands = [np.nextafter(c, np.float32(-1)), c, np.nextafter(c, np.float32(2))]
    return float(min(cands, key=lambda v: abs(Fraction(float(v)) - x)))


def test_sah_factor_table():
    # sahFactorConfigSse.txt rows; N and L rounded up to the gang of 4.
    assert pkg.sah_factor(4, 4) == _stof("0.9790158394920848")
    assert pkg.sah_factor(8, 8) == _stof("0.8089449478051558")
    assert pkg.sah_factor(16, 16) == _stof("0.7655054621988963")
    assert pkg.sah_factor(12, 4) == _stof("1.5611955563121058")
    assert pkg.sah_factor(3, 2) == pkg.sah_factor(4, 4)
    assert pkg.sah_factor(9, 5) == pkg.sah_factor(12, 8)
    assert pkg.sah_factor(8, 8, gang=8) == 1.0


def test_struct_layouts_match_the_c_header(tmp_path):
    """The ctypes mirrors have the sizes and field offsets the C compiler
    gives the header's structs."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [("bvhgpu_build_params_t", N.BuildParams), ("bvhgpu_bvh_info_t", N.BvhInfo),
             ("bvhgpu_scene_params_t", N.SceneParams), ("bvhgpu_trace_opts_t", N.TraceOpts),
             ("bvhgpu_batch_t", N.Batch), ("bvhgpu_job_t", N.Job),
             ("bvhgpu_host_batch_t", N.HostBatch),
             ("bvhgpu_camera_t", N.Camera), ("bvhgpu_secondary_t", N.Secondary)]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "bvhgpu.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parents[1] / "include"
    subprocess.run([cc, "-std=c11", f"-I{inc}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for cname, py in pairs:
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])


def test_new_entry_points_validate_arguments_without_a_gpu():
    """Argument checks of the batched ISPC calls, the multi-batch host trace
    and the stored-hit adjoint run before any device work."""
    lib = N.lib()
    assert lib.bvhgpu_gang_size() == 4
    buf = np.zeros(64, np.float32)
    ids = np.zeros(1, np.uint32)
    res = np.zeros(4, np.uint8)
    assert lib.bvhgpu_aabb_intersect(5, buf.ctypes.data, ids.ctypes.data, buf.ctypes.data,
                                     buf.ctypes.data, res.ctypes.data, 1, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_aabb_intersect(8, None, None, None, None, None, 0, None) == N.OK
    assert lib.bvhgpu_aabb_intersect(8, None, ids.ctypes.data, buf.ctypes.data,
                                     buf.ctypes.data, res.ctypes.data, 1, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_tri_intersect(8, 3, buf.ctypes.data, ids.ctypes.data, buf.ctypes.data,
                                    res.ctypes.data, 1, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_tri_intersect(7, 4, buf.ctypes.data, ids.ctypes.data, buf.ctypes.data,
                                    res.ctypes.data, 1, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_tri_any_hit(20, buf.ctypes.data, ids.ctypes.data, buf.ctypes.data,
                                  res.ctypes.data, 1, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_trace_host_batches(None, None, 1, None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_adjoint_hits(None, None, None, 1, None, None, None, None, 0, 0, None,
                                   None, None, None) == N.ERR_BAD_ARG
    assert b"null" in lib.bvhgpu_last_error()


def test_noalloc_entry_point_rejects_bad_arguments_without_a_gpu():
    """bvhgpu_trace_batches_noalloc checks its batches and options before any
    CUDA call. The scene handle is a zeroed host buffer: none of these checks
    reads it."""
    lib = N.lib()
    fake_scene = C.create_string_buffer(4096)
    rays = np.zeros((4, 8), np.float32)
    hits = np.zeros((4, 4), np.float32)
    occ = np.zeros(4, np.uint8)
    o = N.TraceOpts(0, 2, 0, 16, 128, 0, 0, 0, 0, 0, 0)

    def call(batches, n=None, opts=o):
        arr = (N.Batch * max(1, len(batches)))(*batches)
        return lib.bvhgpu_trace_batches_noalloc(fake_scene, arr,
                                                len(batches) if n is None else n,
                                                C.byref(opts) if opts is not None else None, None)

    good = N.Batch(rays.ctypes.data, 4, N.CLOSEST, 0, hits.ctypes.data, None)
    assert call([good] * 65) == N.ERR_BAD_ARG  # more heads than the fixed scratch holds
    assert b"64" in lib.bvhgpu_last_error()
    assert lib.bvhgpu_trace_batches_noalloc(fake_scene, None, 1, C.byref(o), None) == N.ERR_BAD_ARG
    assert lib.bvhgpu_trace_batches_noalloc(None, None, 0, C.byref(o), None) == N.ERR_BAD_ARG
    assert call([good], opts=None) == N.ERR_BAD_ARG
    assert call([N.Batch(rays.ctypes.data, 4, 7, 0, hits.ctypes.data, None)]) == N.ERR_BAD_ARG
    assert b"kind" in lib.bvhgpu_last_error()
    assert call([N.Batch(rays.ctypes.data + 4, 4, N.CLOSEST, 0, hits.ctypes.data, None)]) \
        == N.ERR_BAD_ARG
    assert call([N.Batch(None, 4, N.CLOSEST, 0, hits.ctypes.data, None)]) == N.ERR_BAD_ARG
    assert call([N.Batch(rays.ctypes.data, 4, N.CLOSEST, 0, hits.ctypes.data + 8, None)]) \
        == N.ERR_BAD_ARG
    assert call([N.Batch(rays.ctypes.data, 4, N.ANY, 0, None, None)]) == N.ERR_BAD_ARG
    assert call([N.Batch(rays.ctypes.data, 1 << 41, N.ANY, 0, None, occ.ctypes.data)]) \
        == N.ERR_BAD_ARG
    for bad in (N.TraceOpts(0, 2, 0, 16, 128, 0, 0, 0, 10, 0, 0),   # reorder
                N.TraceOpts(0, 0, 0, 16, 128, 0, 0, 1, 0, 0, 0),    # save_distance
                N.TraceOpts(0, 0, 0, 16, 128, 0, 0, 0, 0, 1, 0)):   # stack_local
        assert call([good], opts=bad) == N.ERR_UNSUPPORTED
    assert call([good], opts=N.TraceOpts(0, 2, 0, 16, 128, 5, 0, 0, 0, 0, 0)) == N.ERR_BAD_ARG


def test_noalloc_python_binding_rejects_mismatched_buffers():
    """The binding checks shapes, dtypes, contiguity and devices before the
    call, since the kernel writes n records into ``out`` unchecked."""
    torch = pytest.importorskip("torch")
    check = pkg.check_noalloc_batch
    rays = torch.zeros((6, 8), dtype=torch.float32)
    check(rays, "closest", torch.zeros((6, 4), dtype=torch.float32), "cpu")
    check(rays, "any", torch.zeros(6, dtype=torch.uint8), "cpu")
    bad = [
        (rays, "closest", torch.zeros((5, 4), dtype=torch.float32)),       # too few rows
        (rays, "closest", torch.zeros((6, 4), dtype=torch.float64)),       # dtype
        (rays, "any", torch.zeros(5, dtype=torch.uint8)),                  # too few bytes
        (rays, "any", torch.zeros((6, 4), dtype=torch.float32)),           # any-hit as closest
        (rays, "closest", torch.zeros((4, 6), dtype=torch.float32).t()),   # strided out
        (torch.zeros((8, 6), dtype=torch.float32).t(), "closest",
         torch.zeros((6, 4), dtype=torch.float32)),                        # strided rays
        (torch.zeros((6, 8), dtype=torch.float64), "closest",
         torch.zeros((6, 4), dtype=torch.float32)),                        # ray dtype
        (torch.zeros((6, 7), dtype=torch.float32), "closest",
         torch.zeros((6, 4), dtype=torch.float32)),                        # ray width
        (rays, "nearest", torch.zeros((6, 4), dtype=torch.float32)),       # kind
    ]
    for r, k, o in bad:
        with pytest.raises(ValueError):
            check(r, k, o, "cpu")
    with pytest.raises(ValueError):  # buffers on another device than the scene
        check(rays, "closest", torch.zeros((6, 4), dtype=torch.float32), "cuda:0")


def test_read_bandwidth_rejects_bad_arguments_without_a_gpu():
    lib = N.lib()
    g = C.c_double()
    assert lib.bvhgpu_read_bandwidth(0, 1024, 1, 1, C.byref(g)) == N.ERR_BAD_ARG
    assert lib.bvhgpu_read_bandwidth(0, 1 << 20, 0, 1, C.byref(g)) == N.ERR_BAD_ARG
    assert lib.bvhgpu_read_bandwidth(0, 1 << 20, 1, 1, None) == N.ERR_BAD_ARG
