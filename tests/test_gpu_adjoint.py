"""Adjoint of the leaf intersection (bvhgpu_adjoint) behind torch.autograd:
checked against PyTorch autograd of Moller-Trumbore on the same hit set and
against central finite differences in FP64 (h = 1e-4)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from bvhraytracer_gb300 import diff as D  # noqa: E402
from bvhraytracer_gb300 import scenes as S  # noqa: E402

pytestmark = pytest.mark.gpu


def _case(n=64, res=96, seed=0):
    verts, faces = S.terrain_mesh(n, seed)
    c = np.array([0.5, 0.0, 0.5])
    rays = S.camera_rays(c + [0.0, 0.6, 0.7], c, res, res)
    v = torch.from_numpy(verts).cuda().requires_grad_(True)
    f = torch.from_numpy(faces).cuda()
    r = torch.from_numpy(rays).cuda().requires_grad_(True)
    scene = D.scene_for(v, f)
    # targets from vertices moved by seeded N(0, 0.01) noise
    rng = np.random.default_rng(seed + 1)
    vt = torch.from_numpy(verts + rng.normal(0, 0.01, verts.shape).astype(np.float32)).cuda()
    t_tgt, _, _, p_tgt = D.ray_hit(vt, f, r.detach(), D.scene_for(vt, f))
    return v, f, r, scene, t_tgt, p_tgt


def _loss_and_grads(v, f, r, scene, t_tgt, p_tgt):
    t, u, w, prim = D.ray_hit(v, f, r, scene)
    m = (prim >= 0) & (p_tgt >= 0)
    loss = ((t - t_tgt)[m] ** 2).sum()
    gv, gr = torch.autograd.grad(loss, (v, r))
    return loss, gv, gr, prim, m


def test_adjoint_matches_torch_autograd_moller_trumbore():
    v, f, r, scene, t_tgt, p_tgt = _case()
    loss, gv, gr, prim, m = _loss_and_grads(v, f, r, scene, t_tgt, p_tgt)
    # Same loss with PyTorch autograd of Moller-Trumbore on the same hit set.
    v2 = v.detach().clone().requires_grad_(True)
    r2 = r.detach().clone().requires_grad_(True)
    idx = torch.nonzero(m).squeeze(1)
    tri = f[prim[idx].long()]
    t2, b1, b2 = D.moller_trumbore_torch(r2[idx, 0:3], r2[idx, 4:7], v2[tri[:, 0]],
                                         v2[tri[:, 1]], v2[tri[:, 2]])
    t_fwd, u_fwd, w_fwd, _ = D.ray_hit(v, f, r, scene)
    # the same forward values (torch may contract to FMA, so not bit for bit)
    assert torch.allclose(t2.detach(), t_fwd[idx].detach(), rtol=1e-5, atol=0)
    loss2 = ((t2 - t_tgt[idx]) ** 2).sum()
    gv2, gr2 = torch.autograd.grad(loss2, (v2, r2))
    rel_v = (gv - gv2).norm() / gv2.norm()
    rel_r = (gr[:, [0, 1, 2, 4, 5, 6]] - gr2[:, [0, 1, 2, 4, 5, 6]]).norm() / gr2.norm()
    # two FP32 evaluations in different operation orders (atomics, FMA in
    # torch): agreement to ~1e-5 of the gradient norm
    assert rel_v < 1e-4 and rel_r < 1e-4, (rel_v.item(), rel_r.item())


@pytest.mark.parametrize("which", ["t", "uv"])
def test_recompute_backward_equals_stored_hits(which):
    """ray_hit(recompute=True) re-traces in the backward pass instead of
    keeping the forward's hits: the same per-ray gradients bit for bit, the
    same vertex gradients up to the order of the atomic sums."""
    v, f, r, scene, t_tgt, p_tgt = _case(n=48, res=80, seed=3)
    out = []
    for recompute in (False, True):
        t, u, w, prim = D.ray_hit(v, f, r, scene, recompute=recompute)
        m = (prim >= 0) & (p_tgt >= 0)
        if which == "t":
            loss = torch.where(m, (t - t_tgt) ** 2, torch.zeros_like(t)).sum()
        else:
            loss = torch.where(m, 0.7 * u - 1.3 * w, torch.zeros_like(u)).sum()
        out.append(torch.autograd.grad(loss, (v, r)))
    (gv0, gr0), (gv1, gr1) = out
    scene.status()
    assert torch.equal(gr0, gr1)
    assert gv0.abs().max() > 0
    assert (gv0 - gv1).abs().max() <= 1e-5 * gv0.abs().max()


def test_non_contiguous_rays():
    """Rays given as a strided view (8 of 11 columns): the same hits and
    gradients as the contiguous copy, in both backward modes."""
    v, f, r, scene, t_tgt, p_tgt = _case(n=32, res=48, seed=5)
    wide = torch.zeros((r.shape[0], 11), dtype=torch.float32, device="cuda")
    wide[:, 2:10] = r.detach()
    rs = wide[:, 2:10].requires_grad_(True)
    assert not rs.is_contiguous()
    for recompute in (False, True):
        got, want = [], []
        for rays, out in ((rs, got), (r, want)):
            t, u, w, prim = D.ray_hit(v, f, rays, scene, recompute=recompute)
            loss = torch.where(prim >= 0, t + 0.5 * u, torch.zeros_like(t)).sum()
            out.append((t.detach(), prim) + torch.autograd.grad(loss, (v, rays)))
        assert torch.equal(got[0][0], want[0][0]) and torch.equal(got[0][1], want[0][1])
        assert torch.equal(got[0][3], want[0][3])
        assert (got[0][2] - want[0][2]).abs().max() <= 1e-5 * want[0][2].abs().max()
    scene.status()


def test_adjoint_matches_fp64_chain_rule():
    """The reverse pass against float64 PyTorch autograd of Moller-Trumbore on
    the CPU, fed the same upstream gradient (from the FP32 forward t): with
    the double-float reverse pass the two agree to FP32 accumulation error,
    grazing rays included."""
    v, f, r, scene, t_tgt, p_tgt = _case(n=64, res=128)
    loss, gv, gr, prim, m = _loss_and_grads(v, f, r, scene, t_tgt, p_tgt)
    t, _, _, _ = D.ray_hit(v, f, r, scene)
    idx = torch.nonzero(m).squeeze(1)
    up = (2 * (t.detach() - t_tgt))[idx].double().cpu()
    V = v.detach().double().cpu().requires_grad_(True)
    R = r.detach().double().cpu()[idx.cpu()].requires_grad_(True)
    tri = f.cpu()[prim[idx].long().cpu()]
    t64, _, _ = D.moller_trumbore_torch(R[:, 0:3], R[:, 4:7], V[tri[:, 0]], V[tri[:, 1]],
                                        V[tri[:, 2]])
    g_v, g_r = torch.autograd.grad(t64, (V, R), grad_outputs=up)
    rel_v = (gv.double().cpu() - g_v).norm() / g_v.norm()
    gr_hit = gr.double().cpu()[idx.cpu()][:, [0, 1, 2, 4, 5, 6]]
    rel_r = (gr_hit - g_r[:, [0, 1, 2, 4, 5, 6]]).norm() / g_r.norm()
    assert rel_v < 1e-5 and rel_r < 1e-5, (rel_v.item(), rel_r.item())


def test_adjoint_barycentric_gradients():
    """Gradients through the barycentrics against float64 PyTorch autograd of
    Moller-Trumbore on the CPU (same hits, same upstream weights)."""
    v, f, r, scene, t_tgt, p_tgt = _case(n=32, res=48)
    t, u, w, prim = D.ray_hit(v, f, r, scene)
    m = prim >= 0
    loss = (u[m] * 0.7 - w[m] * 1.3).sum()
    gv, = torch.autograd.grad(loss, (v,))
    idx = torch.nonzero(m).squeeze(1).cpu()
    V = v.detach().double().cpu().requires_grad_(True)
    R = r.detach().double().cpu()[idx]
    tri = f.cpu()[prim[m].long().cpu()]
    _, b1, b2 = D.moller_trumbore_torch(R[:, 0:3], R[:, 4:7], V[tri[:, 0]], V[tri[:, 1]],
                                        V[tri[:, 2]])
    g64, = torch.autograd.grad((b1 * 0.7 - b2 * 1.3).sum(), (V,))
    assert (gv.double().cpu() - g64).norm() / g64.norm() < 1e-5


def _fd_loss(o, d, p0, p1, p2, tgt):
    """FP64 loss over fixed ray/triangle pairs (numpy)."""
    e1 = p1 - p0
    e2 = p2 - p0
    s1 = np.cross(d, e2)
    inv = 1.0 / np.sum(s1 * e1, -1)
    s = o - p0
    s2 = np.cross(s, e1)
    t = np.sum(e2 * s2, -1) * inv
    return np.sum((t - tgt) ** 2)


def test_adjoint_against_fp64_finite_differences():
    """FP64 central differences on 512 sampled vertex coordinates and on the
    origin / direction of 128 sampled rays. At h = 1e-4 the differences
    themselves are off by about 1% on rays that graze steep triangles (t is
    a rational function of the vertices); they converge to the adjoint as h
    shrinks, so the check uses h = 1e-6 and a Richardson extrapolation of
    h = 1e-4 and 5e-5."""
    v, f, r, scene, t_tgt, p_tgt = _case(n=64, res=128)
    loss, gv, gr, prim, m = _loss_and_grads(v, f, r, scene, t_tgt, p_tgt)
    V = v.detach().cpu().numpy().astype(np.float64)
    F = f.cpu().numpy()
    R = r.detach().cpu().numpy().astype(np.float64)
    P = prim.cpu().numpy()
    M = m.cpu().numpy()
    T = t_tgt.cpu().numpy().astype(np.float64)
    rays_hit = np.nonzero(M)[0]
    tri_of = P[rays_hit]
    touched = np.unique(F[tri_of].reshape(-1))
    rng = np.random.default_rng(3)
    vids = rng.choice(touched, 512, replace=True)
    axes = rng.integers(0, 3, 512)
    gad = gv.cpu().numpy().astype(np.float64)

    def fd_vertex(vid, ax, h):
        sel = np.any(F[tri_of] == vid, axis=1)
        rr = rays_hit[sel]
        tt = F[P[rr]]

        def L(delta):
            W = V.copy()
            W[vid, ax] += delta
            return _fd_loss(R[rr, 0:3], R[rr, 4:7], W[tt[:, 0]], W[tt[:, 1]], W[tt[:, 2]], T[rr])
        return (L(h) - L(-h)) / (2 * h)

    ad = gad[vids, axes]
    fd = {h: np.array([fd_vertex(a, b, h) for a, b in zip(vids, axes)])
          for h in (1e-4, 5e-5, 1e-6)}
    rich = (4 * fd[5e-5] - fd[1e-4]) / 3

    def rel(x):
        return np.linalg.norm(ad - x) / np.linalg.norm(x)
    assert rel(fd[1e-6]) < 1e-4, rel(fd[1e-6])
    assert rel(rich) < 1e-3, rel(rich)
    assert rel(fd[1e-4]) < 5e-2  # truncation-limited, reported by the adjoint bench
    # ray origin / direction gradients on 128 sampled rays
    pick = rng.choice(rays_hit, 128, replace=False)
    gR = gr.cpu().numpy().astype(np.float64)
    fdr, adr = [], []
    for i in pick:
        tri = F[P[i]]
        for comp in (0, 1, 2, 4, 5, 6):
            def Lr(delta):
                Q = R[i].copy()
                Q[comp] += delta
                return _fd_loss(Q[None, 0:3], Q[None, 4:7], V[tri[0]][None], V[tri[1]][None],
                                V[tri[2]][None], T[i:i + 1])
            fdr.append((Lr(1e-6) - Lr(-1e-6)) / 2e-6)
            adr.append(gR[i, comp])
    fdr, adr = np.array(fdr), np.array(adr)
    assert np.linalg.norm(adr - fdr) / np.linalg.norm(fdr) < 1e-4


def test_per_triangle_and_per_vertex_entry_points_agree():
    """bvhgpu_adjoint (per-triangle gradients, scattered by the caller) and
    bvhgpu_adjoint_vertices (accumulated through the face indices) give the
    same vertex gradients; out-of-range vertex ids are reported, not written."""
    import ctypes as C
    from bvhraytracer_gb300 import _native as N
    v, f, r, scene, t_tgt, p_tgt = _case(n=32, res=64)
    n = r.shape[0]
    gh = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    gh[:, 1] = torch.linspace(-1, 1, n, device="cuda")
    gh[:, 2] = 0.3
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    tri9 = torch.zeros((f.shape[0], 9), dtype=torch.float32, device="cuda")
    gr1 = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    rays = r.detach().contiguous()
    N.check(N.lib().bvhgpu_adjoint(scene.handle, rays.data_ptr(), n, gh.data_ptr(),
                                   tri9.data_ptr(), gr1.data_ptr(), st))
    gv1 = torch.zeros((v.shape[0], 3), dtype=torch.float32, device="cuda")
    gv1.index_add_(0, f.reshape(-1), tri9.view(-1, 3))
    f32 = f.to(torch.int32).contiguous()
    gv2 = torch.zeros_like(gv1)
    gr2 = torch.empty_like(gr1)
    N.check(N.lib().bvhgpu_adjoint_vertices(scene.handle, rays.data_ptr(), n, gh.data_ptr(),
                                            f32.data_ptr(), f32.shape[0], v.shape[0],
                                            gv2.data_ptr(), gr2.data_ptr(), st))
    torch.cuda.synchronize()
    assert torch.equal(gr1, gr2)
    assert (gv1 - gv2).abs().max() <= 1e-5 * gv1.abs().max()
    bad = f32.clone()
    bad[:] = v.shape[0] + 5
    gv3 = torch.zeros_like(gv1)
    N.check(N.lib().bvhgpu_adjoint_vertices(scene.handle, rays.data_ptr(), n, gh.data_ptr(),
                                            bad.data_ptr(), bad.shape[0], v.shape[0],
                                            gv3.data_ptr(), gr2.data_ptr(), st))
    with pytest.raises(Exception):
        scene.status()
    assert torch.count_nonzero(gv3) == 0


def test_adjoint_from_stored_hits_equals_retrace():
    """bvhgpu_adjoint_hits (the forward pass's hits, no traversal) gives the
    re-tracing entry points' ray gradients bit for bit and their triangle /
    vertex gradients up to the order of the atomic sums; misses and inactive
    rays get zero gradients; a triangle id the scene does not hold is
    reported and skipped."""
    import ctypes as C
    from bvhraytracer_gb300 import _native as N
    v, f, r, scene, t_tgt, p_tgt = _case(n=32, res=64, seed=3)
    rays = r.detach().clone()
    rays[::53, 0] = float("nan")
    rays[7, 4:7] = torch.tensor([0.0, 1.0, 0.0], device="cuda")  # points away: a miss
    rays = rays.contiguous()
    n = rays.shape[0]
    hits = scene.trace(rays, profile="fast")["hits"]
    gh = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    gh[:, 1] = torch.linspace(-1, 1, n, device="cuda")
    gh[:, 2] = 0.3
    gh[:, 3] = -0.2
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    f32 = f.to(torch.int32).contiguous()
    tri_a = torch.zeros((f.shape[0], 9), dtype=torch.float32, device="cuda")
    tri_b = torch.zeros_like(tri_a)
    gr_a = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    gr_b = torch.full_like(gr_a, 7.0)
    N.check(N.lib().bvhgpu_adjoint(scene.handle, rays.data_ptr(), n, gh.data_ptr(),
                                   tri_a.data_ptr(), gr_a.data_ptr(), st))
    # the incoming gradients as separate dL/dt, dL/du, dL/dv arrays
    gtuv = [gh[:, k].contiguous() for k in (1, 2, 3)]
    gp = [x.data_ptr() for x in gtuv]
    N.check(N.lib().bvhgpu_adjoint_hits(scene.handle, rays.data_ptr(), hits.data_ptr(), n,
                                        *gp, None, 0, 0, None, tri_b.data_ptr(),
                                        gr_b.data_ptr(), st))
    gv_a = torch.zeros((v.shape[0], 3), dtype=torch.float32, device="cuda")
    gv_b = torch.zeros_like(gv_a)
    gr_c = torch.empty_like(gr_a)
    N.check(N.lib().bvhgpu_adjoint_vertices(scene.handle, rays.data_ptr(), n, gh.data_ptr(),
                                            f32.data_ptr(), f32.shape[0], v.shape[0],
                                            gv_a.data_ptr(), gr_c.data_ptr(), st))
    N.check(N.lib().bvhgpu_adjoint_hits(scene.handle, rays.data_ptr(), hits.data_ptr(), n,
                                        *gp, f32.data_ptr(), f32.shape[0],
                                        v.shape[0], gv_b.data_ptr(), None, gr_b.data_ptr(), st))
    torch.cuda.synchronize()
    scene.status()
    assert torch.equal(gr_a, gr_b) and torch.equal(gr_a, gr_c)
    assert (tri_a - tri_b).abs().max() <= 1e-5 * tri_a.abs().max()
    assert (gv_a - gv_b).abs().max() <= 1e-5 * gv_a.abs().max()
    miss = hits.view(torch.int32)[:, 0] < 0
    assert bool(miss[7]) and bool(miss[::53].all())
    assert torch.count_nonzero(gr_b[miss]) == 0
    # An id the scene does not hold: zero gradients, reported.
    i = int(torch.nonzero(~miss)[0])
    bad = hits.clone()
    bad.view(torch.int32)[i, 0] = f.shape[0] + 100
    tri_c = torch.zeros_like(tri_a)
    N.check(N.lib().bvhgpu_adjoint_hits(scene.handle, rays[i:].data_ptr(), bad[i:].data_ptr(), 1,
                                        *[x[i:].data_ptr() for x in gtuv], None, 0, 0, None,
                                        tri_c.data_ptr(), gr_b[i:].data_ptr(), st))
    with pytest.raises(Exception):
        scene.status()
    assert torch.count_nonzero(tri_c) == 0 and torch.count_nonzero(gr_b[i]) == 0
    # faces and grad_tri9 together, or neither: rejected on the host
    assert N.lib().bvhgpu_adjoint_hits(scene.handle, rays.data_ptr(), hits.data_ptr(), n,
                                       *gp, f32.data_ptr(), f32.shape[0], v.shape[0],
                                       gv_b.data_ptr(), tri_b.data_ptr(), gr_b.data_ptr(),
                                       st) == N.ERR_BAD_ARG
    assert N.lib().bvhgpu_adjoint_hits(scene.handle, rays.data_ptr(), hits.data_ptr(), n,
                                       *gp, None, 0, 0, None, None, gr_b.data_ptr(),
                                       st) == N.ERR_BAD_ARG


def test_adjoint_many_rays_on_one_triangle():
    """4,096 rays on one large triangle (every lane of every warp has the
    same hit, so the gradients are summed within warps before the atomics):
    the vertex gradients equal FP64 autograd of Moller-Trumbore."""
    import ctypes as C
    from bvhraytracer_gb300 import _native as N
    verts = np.array([[-3, -3, 0], [5, -3, 0], [-3, 5, 0],
                      [5, 5, 1], [6, 5, 1], [5, 6, 1]], np.float32)
    faces = np.array([[0, 1, 2], [3, 4, 5]], np.int64)
    v = torch.from_numpy(verts).cuda()
    f = torch.from_numpy(faces).cuda()
    scene = D.scene_for(v, f, branching=4, leaf_size=4)
    g = np.linspace(-0.9, 0.9, 64, dtype=np.float32)
    xs, ys = np.meshgrid(g, g)
    n = xs.size
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0], rays[:, 1], rays[:, 2] = xs.ravel(), ys.ravel(), 2.0
    rays[:, 3] = 100.0
    rays[:, 4] = 0.05 * xs.ravel()
    rays[:, 5] = -0.03
    rays[:, 6] = -1.0
    r = torch.from_numpy(rays).cuda()
    hits = scene.trace(r, profile="fast")["hits"]
    assert bool((hits.view(torch.int32)[:, 0] == 0).all())
    w = torch.linspace(-1, 2, n, device="cuda")
    gh = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    gh[:, 1] = w
    gh[:, 2] = 0.25 * w
    f32 = f.to(torch.int32).contiguous()
    gv = torch.zeros((6, 3), dtype=torch.float32, device="cuda")
    gr = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # dL/dt and dL/du only: dL/dv passed as NULL (zero)
    gtw, guw = gh[:, 1].contiguous(), gh[:, 2].contiguous()
    N.check(N.lib().bvhgpu_adjoint_hits(scene.handle, r.data_ptr(), hits.data_ptr(), n,
                                        gtw.data_ptr(), guw.data_ptr(), None, f32.data_ptr(), 2,
                                        6, gv.data_ptr(), None, gr.data_ptr(), st))
    gv2 = torch.zeros_like(gv)
    N.check(N.lib().bvhgpu_adjoint_vertices(scene.handle, r.data_ptr(), n, gh.data_ptr(),
                                            f32.data_ptr(), 2, 6, gv2.data_ptr(),
                                            gr.data_ptr(), st))
    torch.cuda.synchronize()
    scene.status()
    p = torch.from_numpy(verts.astype(np.float64)).requires_grad_(True)
    rd = torch.from_numpy(rays.astype(np.float64))
    t, b1, _ = D.moller_trumbore_torch(rd[:, 0:3], rd[:, 4:7], p[0].expand(n, 3),
                                       p[1].expand(n, 3), p[2].expand(n, 3))
    wd = w.double().cpu()
    (gp,) = torch.autograd.grad((t * wd).sum() + (b1 * 0.25 * wd).sum(), (p,))
    ref = gp.numpy()
    for got in (gv, gv2):
        got = got.double().cpu().numpy()
        # float sums of 4,096 terms (a lost term would be ~2.4e-4 of the total)
        assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max(), (got, ref)
        assert np.all(got[3:] == 0)


@pytest.mark.parametrize("name", ["terrain256", "clutter1M"])
def test_adjoint_on_the_differentiation_workload_scenes(name):
    """The differentiation workload's scenes at full size (terrain 256 x 256
    quads, the 1M-triangle clutter scene; 1M primary rays; targets from
    vertices moved by N(0, 0.01)): on 512 sampled vertex coordinates the
    FP32 adjoint is within 1e-4 (norm-relative) of the exact FP64 gradient of
    the same loss and of FP64 central differences at h = 1e-6. At h = 1e-4
    the differences are themselves off the exact gradient (grazing rays make
    t strongly curved in the vertices), by more than the adjoint is; the
    bench reports every step size."""
    import bench
    rng = np.random.default_rng(11)
    if name == "terrain256":
        verts, faces = S.terrain_mesh(256, seed=0)
        c = np.array([0.5, 0.0, 0.5])
        rays = S.camera_rays(c + [0.0, 0.55, 0.65], c, 1024, 1024)
    else:
        tris = S.clutter(4000, seed=1)
        verts = tris.reshape(-1, 3)
        faces = np.arange(verts.shape[0], dtype=np.int64).reshape(-1, 3)
        cam, target, _ = S.clutter_viewpoints(4000, seed=1)
        rays = S.camera_rays(cam, target, 1024, 1024)
    v = torch.from_numpy(verts).cuda().requires_grad_(True)
    f = torch.from_numpy(faces.astype(np.int32)).cuda()
    r = torch.from_numpy(rays).cuda().requires_grad_(True)
    scene = D.scene_for(v, f)
    vt = torch.from_numpy(verts + rng.normal(0, 0.01, verts.shape).astype(np.float32)).cuda()
    t_tgt, _, _, p_tgt = D.ray_hit(vt, f, r.detach(), D.scene_for(vt, f))
    t, u, w, prim = D.ray_hit(v, f, r, scene)
    m = (prim >= 0) & (p_tgt >= 0)
    loss = torch.where(m, (t - t_tgt) ** 2, torch.zeros_like(t)).sum()
    gv, gr = torch.autograd.grad(loss, (v, r))
    res = bench.fd_check(verts, faces, rays, prim.cpu().numpy(), m.cpu().numpy(),
                         t_tgt.cpu().numpy().astype(np.float64), gv.cpu().numpy())
    scene.status()
    assert res["fp64_autograd"] < 1e-4, res
    assert res["h=1e-6"] < 1e-4, res
    trunc = res["fd_truncation_vs_fp64_autograd"]
    assert trunc["h=1e-4"] >= res["fp64_autograd"], res
