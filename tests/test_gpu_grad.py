"""Gradients of the differentiable queries (no counterpart in the reference:
checked against FP64 central finite differences with eps = 1e-4 on 1,024
samples and against an analytic per-primitive FP64 gradient)."""
import numpy as np
import pytest

import fcpw_gb300 as F
from fcpw_gb300 import records as R
from fcpw_gb300 import workloads as W
from helpers import build_scene
from oracle import oracle as O

pytestmark = pytest.mark.gpu
EPS = 1e-4


def _prims_from(v, f):
    p = np.zeros(len(f), R.TRIANGLE)
    p["pa"], p["pb"], p["pc"] = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    p["index"] = np.arange(len(f))
    return p


def _d64(v, f, pts):
    d, idx = O.closest_points_brute_f64(3, _prims_from(v, f), R.make_spheres(pts, R.FLT_MAX))
    return d, idx


@pytest.fixture(scope="module")
def setup():
    import torch
    v, f = W.perturbed_sphere(16, W.SEED_BASE + 4)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    g.set_traversal(4, 8, precise=True)
    x = W.uniform_points(1024, 3, -1.5, 1.5, 51)
    return v, f, g, torch.from_numpy(x).cuda(), torch.from_numpy(v).cuda()


def test_distance_grad_x_matches_fp64_finite_differences(setup):
    import torch
    from fcpw_gb300.autograd import closest_point_distance
    v, f, g, x, vt = setup
    xx = x.clone().requires_grad_(True)
    d = closest_point_distance(g, xx, vt, refit=False)
    d.sum().backward()
    gx = xx.grad.cpu().numpy().astype(np.float64)
    pts = x.cpu().numpy().astype(np.float64)
    fd = np.zeros_like(gx)
    for a in range(3):
        e = np.zeros(3)
        e[a] = EPS
        dp, _ = _d64(v, f, (pts + e).astype(np.float32))
        dm, _ = _d64(v, f, (pts - e).astype(np.float32))
        # the query shift is rounded to float32: divide by the step actually taken
        step = (pts + e).astype(np.float32).astype(np.float64)[:, a] - (pts - e).astype(np.float32).astype(np.float64)[:, a]
        fd[:, a] = (dp - dm) / step
    err = np.linalg.norm(gx - fd, axis=1)
    # distance is smooth away from the medial axis; a few samples sit within eps of it
    assert np.mean(err < 1e-3) > 0.98, np.sort(err)[-10:]
    assert np.allclose(np.linalg.norm(gx, axis=1), 1.0, atol=1e-5)


def test_distance_grad_vertices_match_analytic_fp64(setup):
    import torch
    from fcpw_gb300.autograd import closest_point_distance
    v, f, g, x, vt = setup
    vv = vt.clone().requires_grad_(True)
    d = closest_point_distance(g, x, vv, refit=True)
    (d * d).mean().backward()
    gv = vv.grad.cpu().numpy().astype(np.float64)
    # analytic FP64: dL/dv_k = sum_q (2 d_q / N) * (-b_k) (x_q - p_q) / d_q on q's closest triangle
    pts = x.cpu().numpy().astype(np.float64)
    d64, idx = _d64(v, f, pts.astype(np.float32))
    ref = np.zeros_like(gv)
    vd = v.astype(np.float64)
    for q in range(len(pts)):
        tri = f[idx[q]]
        a, b, c = vd[tri[0]], vd[tri[1]], vd[tri[2]]
        # barycentrics of the FP64 closest point (projection, clamped via the region method)
        p, w = _closest_tri64(a, b, c, pts[q])
        u = (pts[q] - p) / d64[q]
        coef = 2.0 * d64[q] / len(pts)
        for k in range(3):
            ref[tri[k]] -= coef * w[k] * u
    scale = np.abs(ref).max()
    assert np.abs(gv - ref).max() <= 1e-4 * scale


def _closest_tri64(a, b, c, x):
    ab, ac, ax = b - a, c - a, x - a
    d1, d2 = ab @ ax, ac @ ax
    if d1 <= 0 and d2 <= 0:
        return a, (1, 0, 0)
    bx = x - b
    d3, d4 = ab @ bx, ac @ bx
    if d3 >= 0 and d4 <= d3:
        return b, (0, 1, 0)
    cx = x - c
    d5, d6 = ab @ cx, ac @ cx
    if d6 >= 0 and d5 <= d6:
        return c, (0, 0, 1)
    vc = d1 * d4 - d3 * d2
    if vc <= 0 and d1 >= 0 and d3 <= 0:
        t = d1 / (d1 - d3)
        return a + ab * t, (1 - t, t, 0)
    vb = d5 * d2 - d1 * d6
    if vb <= 0 and d2 >= 0 and d6 <= 0:
        t = d2 / (d2 - d6)
        return a + ac * t, (1 - t, 0, t)
    va = d3 * d6 - d5 * d4
    if va <= 0 and (d4 - d3) >= 0 and (d5 - d6) >= 0:
        t = (d4 - d3) / ((d4 - d3) + (d5 - d6))
        return b + (c - b) * t, (0, 1 - t, t)
    den = 1.0 / (va + vb + vc)
    vv, ww = vb * den, vc * den
    return a + ab * vv + ac * ww, (1 - vv - ww, vv, ww)


def test_distance_grad_vertices_finite_differences(setup):
    import torch
    from fcpw_gb300.autograd import closest_point_distance
    v, f, g, x, vt = setup
    vv = vt.clone().requires_grad_(True)
    d = closest_point_distance(g, x, vv, refit=True)
    d.sum().backward()
    gv = vv.grad.cpu().numpy().astype(np.float64)
    pts = x.cpu().numpy()
    _, idx = _d64(v, f, pts)
    touched = np.unique(f[idx].reshape(-1))
    rng = np.random.default_rng(3)
    for vi in rng.choice(touched, size=12, replace=False):
        qs = np.nonzero((f[idx] == vi).any(axis=1))[0]
        for a in range(3):
            vp, vm = v.astype(np.float64).copy(), v.astype(np.float64).copy()
            vp[vi, a] += EPS
            vm[vi, a] -= EPS
            dp, _ = _d64(vp.astype(np.float32), f, pts[qs])
            dm, _ = _d64(vm.astype(np.float32), f, pts[qs])
            step = np.float64(np.float32(vp[vi, a])) - np.float64(np.float32(vm[vi, a]))
            fd = (dp.sum() - dm.sum()) / step
            assert abs(fd - gv[vi, a]) <= 2e-3 * max(1.0, abs(fd)), (vi, a, fd, gv[vi, a])


def test_vertex_gradients_are_deterministic(setup):
    import torch
    from fcpw_gb300.autograd import closest_point_distance
    v, f, g, x, vt = setup
    grads = []
    for _ in range(3):
        vv = vt.clone().requires_grad_(True)
        d = closest_point_distance(g, x, vv, refit=True)
        (d * d).mean().backward()
        grads.append(vv.grad.cpu().numpy())
    assert grads[0].tobytes() == grads[1].tobytes() == grads[2].tobytes()


def test_ray_hit_gradients_match_fp64_finite_differences():
    import torch
    from fcpw_gb300.autograd import ray_hit_distance
    v, f = W.perturbed_sphere(16, W.SEED_BASE + 9)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    n = 512
    o = W.uniform_points(n, 3, -0.3, 0.3, 52)  # inside the sphere: every ray hits
    dirs = W.uniform_directions(n, 3, 53)
    ot = torch.from_numpy(o).cuda().requires_grad_(True)
    dt = torch.from_numpy(dirs).cuda().requires_grad_(True)
    vt = torch.from_numpy(v).cuda().requires_grad_(True)
    t = ray_hit_distance(g, ot, dt, vt, refit=False)
    assert torch.isfinite(t).all()
    t.sum().backward()
    go = ot.grad.cpu().numpy().astype(np.float64)
    prims = _prims_from(v, f)

    def t64(oo, dd):
        tt, _ = O.intersect_rays_brute_f64(3, prims, R.make_rays(oo.astype(np.float32), dd.astype(np.float32), R.FLT_MAX))
        return tt
    for a in range(3):
        e = np.zeros(3)
        e[a] = EPS
        fd = (t64(o + e, dirs) - t64(o - e, dirs)) / (np.float32(o[:, a] + EPS).astype(np.float64) - np.float32(o[:, a] - EPS).astype(np.float64))
        ok = np.abs(go[:, a] - fd) <= 2e-3 * np.maximum(1.0, np.abs(fd))
        assert ok.mean() > 0.98
    # vertex gradients sum to minus the origin gradient summed over all rays (translation invariance)
    assert np.allclose(vt.grad.sum(0).cpu().numpy(), -ot.grad.sum(0).cpu().numpy(), rtol=1e-3, atol=1e-3)


def test_optimisation_with_gpu_refit_reduces_loss_and_stays_consistent():
    import torch
    from fcpw_gb300.autograd import closest_point_distance
    v, f = W.perturbed_sphere(16, W.SEED_BASE + 10)
    s = build_scene(3, v, f)
    g = F.GPUScene3D()
    g.transfer_to_gpu(s)
    g.set_traversal(4, 8)
    target = torch.from_numpy(W.uniform_points(4096, 3, -0.6, 0.6, 54)).cuda()
    verts = torch.from_numpy(v).cuda().requires_grad_(True)
    opt = torch.optim.SGD([verts], lr=20.0)
    losses = []
    for _ in range(8):
        opt.zero_grad()
        d = closest_point_distance(g, target, verts, refit=True)
        loss = (d * d).mean()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < losses[0]
    # after the last refit the GPU tree answers like a host tree built on the moved vertices
    vnow = verts.detach().cpu().numpy()
    g.update_vertices_tensor(verts.detach().contiguous())
    out = F.GPUInteractionList()
    pts = target.cpu().numpy()
    g.find_closest_points(pts, np.full(len(pts), R.FLT_MAX, np.float32), out)
    d64, _ = _d64(vnow, f, pts)
    assert np.allclose(out.array()["d"], d64, rtol=1e-6, atol=1e-7)
