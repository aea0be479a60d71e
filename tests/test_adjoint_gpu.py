"""GPU checks of the differentiable closest hit (rdn_attr_loss_forward /
rdn_attr_loss_adjoint): forward values against the oracle's hits, gradients
against an FP64 analytic gradient over all vertices and against FP64 central
differences (h = 1e-4) on 64 random vertices, at frozen visibility."""

import ctypes as C

import numpy as np
import pytest
import torch

from helpers import orc, rt, scenes, single_mesh_scene
from rendiation_gb300 import native

pytestmark = pytest.mark.gpu


class AttrLoss(torch.autograd.Function):
    """Test-harness autograd wrapper: loss(attributes, positions) through the C ABI.
    Positions enter through the acceleration structure, so their gradient is
    returned but the forward ignores the tensor value."""

    @staticmethod
    def forward(ctx, attributes, positions, system, rays, targets, record=False):
        """record: the forward keeps each ray's hit (triangle, instance) and the
        backward differentiates those hits instead of tracing again."""
        L = native.lib()
        n = rays.shape[0]
        loss = torch.zeros(1, dtype=torch.float64, device="cuda")
        hit_tri = torch.zeros(n, dtype=torch.int32, device="cuda")
        hit_inst = torch.zeros(n, dtype=torch.int32, device="cuda")
        d = native.AttrLossDesc(rays.data_ptr(), n, 0, attributes.data_ptr(), targets.data_ptr(), None, None,
                                loss.data_ptr(), None, None, None, 1.0, rt.TRAVERSAL_ORDERED, 0, 0,
                                hit_tri.data_ptr() if record else None, hit_inst.data_ptr() if record else None)
        st = L.rdn_attr_loss_forward(system._h, C.byref(d), C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, L.rdn_last_error(system._h).decode()
        ctx.save_for_backward(attributes, rays, targets, hit_tri, hit_inst)
        ctx.system = system
        ctx.nv = positions.shape[0]
        ctx.record = record
        return loss.to(torch.float32)

    @staticmethod
    def backward(ctx, g):
        attributes, rays, targets, hit_tri, hit_inst = ctx.saved_tensors
        L = native.lib()
        grad = torch.zeros((ctx.nv, 4), dtype=torch.float32, device="cuda")
        rec = ctx.record
        d = native.AttrLossDesc(rays.data_ptr(), rays.shape[0], 0, attributes.data_ptr(), targets.data_ptr(), None,
                                None, None, grad.data_ptr(), None, None, float(g.item()), rt.TRAVERSAL_ORDERED, 0,
                                int(rec), hit_tri.data_ptr() if rec else None, hit_inst.data_ptr() if rec else None)
        st = L.rdn_attr_loss_adjoint(ctx.system._h, C.byref(d), C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, L.rdn_last_error(ctx.system._h).decode()
        return grad[:, 3].contiguous(), grad[:, :3].contiguous(), None, None, None, None


def fp64_hits(pos, idx, rays, tri):
    """FP64 barycentrics of each ray on its (frozen) hit triangle."""
    v = pos.astype(np.float64)[idx.reshape(-1, 3)[tri]]
    o = rays["org"].astype(np.float64)
    d = rays["dir"].astype(np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    s = o - v[:, 0]
    M = np.stack([-d, e1, e2], axis=2)  # columns
    x = np.linalg.solve(M, s[..., None])[..., 0]
    return x[:, 0], x[:, 1], x[:, 2], M


def fp64_loss(pos, idx, attr, rays, tri, targets):
    t, u, v, _ = fp64_hits(pos, idx, rays, tri)
    tv = idx.reshape(-1, 3)[tri]
    val = (1 - u - v) * attr[tv[:, 0]] + u * attr[tv[:, 1]] + v * attr[tv[:, 2]]
    return np.sum((val - targets) ** 2)


@pytest.fixture(scope="module")
def field():
    n = 64
    mesh = scenes.heightfield(n, seed=3)
    rng = np.random.default_rng(5)
    attr = rng.random(mesh.positions.shape[0]).astype(np.float32)
    cam = scenes.PinholeCamera.look_at((0.5, -0.2, 0.9), (0.5, 0.5, 0.0), 35.0, 96, 96)
    rays = scenes.pinhole_rays(cam)
    sc = single_mesh_scene(mesh, bins=4)
    S, P = sc.build_oracle(), sc.build_product()
    hits, _ = S.trace(rays, threads=4)
    return mesh, attr, rays, hits, S, P


def test_forward_matches_oracle_hits(field, cuda):
    mesh, attr, rays, hits, S, P = field
    L = native.lib()
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_attr = torch.from_numpy(attr).cuda()
    value = torch.zeros(rays.shape[0], device="cuda")
    loss = torch.zeros(rays.shape[0], device="cuda")
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    d = native.AttrLossDesc(d_rays.data_ptr(), rays.shape[0], 0, d_attr.data_ptr(), None, value.data_ptr(),
                            loss.data_ptr(), tot.data_ptr(), None, None, None, 1.0, rt.TRAVERSAL_REFERENCE, 0, 0)
    assert L.rdn_attr_loss_forward(P._h, C.byref(d), None) == 0
    torch.cuda.synchronize()
    hit = hits["prim"] != orc.MISS
    tri = hits["prim"][hit]
    tv = mesh.indices.reshape(-1, 3)[tri]
    # the loss kernels re-solve the barycentrics of the traversal's hit in float-float:
    # the value must match the FP64 interpolation on the same triangle
    t64, u64, v64, _ = fp64_hits(mesh.positions, mesh.indices, rays[hit], tri)
    a64 = attr.astype(np.float64)
    expect = (1 - u64 - v64) * a64[tv[:, 0]] + u64 * a64[tv[:, 1]] + v64 * a64[tv[:, 2]]
    got = value.cpu().numpy()
    assert np.max(np.abs(got[hit] - expect)) < 2e-6
    assert np.all(got[~hit] == 0)
    assert abs(tot.item() - float(np.sum(loss.cpu().numpy().astype(np.float64)))) < 1e-6 * max(1.0, tot.item())


@pytest.mark.parametrize("record", [False, True])
def test_gradients_vs_fp64(field, record, cuda):
    """record: the adjoint differentiates the hits the forward recorded."""
    mesh, attr, rays, hits, S, P = field
    rng = np.random.default_rng(9)
    hit = hits["prim"] != orc.MISS
    targets = rng.random(rays.shape[0]).astype(np.float32)
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_attr = torch.from_numpy(attr).cuda().requires_grad_(True)
    d_pos = torch.from_numpy(mesh.positions.copy()).cuda().requires_grad_(True)
    d_tgt = torch.from_numpy(targets).cuda()
    loss = AttrLoss.apply(d_attr, d_pos, P, d_rays, d_tgt, record)
    loss.backward()
    g_attr = d_attr.grad.cpu().numpy().astype(np.float64)
    g_pos = d_pos.grad.cpu().numpy().astype(np.float64)

    # FP64 analytic gradient at frozen visibility (same formulas, double precision)
    tri = hits["prim"][hit]
    rh = rays[hit]
    tg = targets[hit].astype(np.float64)
    t, u, v, M = fp64_hits(mesh.positions, mesh.indices, rh, tri)
    tv = mesh.indices.reshape(-1, 3)[tri]
    a = attr.astype(np.float64)
    val = (1 - u - v) * a[tv[:, 0]] + u * a[tv[:, 1]] + v * a[tv[:, 2]]
    r = 2 * (val - tg)
    g = np.stack([np.zeros_like(r), r * (a[tv[:, 1]] - a[tv[:, 0]]), r * (a[tv[:, 2]] - a[tv[:, 0]])], 1)
    lam = np.linalg.solve(np.transpose(M, (0, 2, 1)), g[..., None])[..., 0]
    ga = np.zeros(a.shape[0])
    gp = np.zeros((a.shape[0], 3))
    for k, wk in enumerate([1 - u - v, u, v]):
        np.add.at(ga, tv[:, k], r * wk)
        np.add.at(gp, tv[:, k], -wk[:, None] * lam)
    # per vertex, against the FP64 analytic gradient
    norm_p = np.linalg.norm(gp, axis=1)
    floor_p = 1e-2 * np.median(norm_p[norm_p > 0])
    floor_a = 1e-2 * np.median(np.abs(ga[ga != 0]))
    rel_p = np.linalg.norm(g_pos - gp, axis=1) / np.maximum(norm_p, floor_p)
    rel_a = np.abs(g_attr - ga) / np.maximum(np.abs(ga), floor_a)
    assert rel_p.max() < 1e-3, rel_p.max()
    assert rel_a.max() < 1e-3, rel_a.max()

    # FP64 central differences on 64 random vertices that some ray sees, with
    # h = 1e-4 and h/2 combined by Richardson extrapolation (error O(h^4)); the
    # difference between the extrapolations at h and h/2 bounds the FD error
    # itself (grazing rays make the barycentrics strongly nonlinear at h = 1e-4)
    seen = np.unique(tv.reshape(-1))
    pick = rng.choice(seen, size=min(64, seen.size), replace=False)
    pos64 = mesh.positions.astype(np.float64)

    def sub_loss(pos, attrs, sel):
        return fp64_loss(pos, mesh.indices, attrs, rh[sel], tri[sel], tg[sel])

    def central(vi, c, hh, sel):
        if c < 3:
            pp, pm = pos64.copy(), pos64.copy()
            pp[vi, c] += hh
            pm[vi, c] -= hh
            return (sub_loss(pp, a, sel) - sub_loss(pm, a, sel)) / (2 * hh)
        ap, am = a.copy(), a.copy()
        ap[vi] += hh
        am[vi] -= hh
        return (sub_loss(pos64, ap, sel) - sub_loss(pos64, am, sel)) / (2 * hh)

    h = 1e-4
    worst_plain, worst = 0.0, 0.0
    for vi in pick:
        sel = np.nonzero(np.any(tv == vi, axis=1))[0]
        fd_h = np.array([central(vi, c, h, sel) for c in range(4)])
        fd_h2 = np.array([central(vi, c, h / 2, sel) for c in range(4)])
        fd_h4 = np.array([central(vi, c, h / 4, sel) for c in range(4)])
        rich = (4 * fd_h2 - fd_h) / 3
        rich2 = (4 * fd_h4 - fd_h2) / 3
        fd_unc = np.linalg.norm(rich[:3] - rich2[:3])
        got = np.array([*g_pos[vi], g_attr[vi]])
        den = max(np.linalg.norm(rich2[:3]), floor_p)
        err = np.linalg.norm(got[:3] - rich2[:3])
        assert err <= 1e-3 * den + 2 * fd_unc, (vi, err / den, fd_unc / den)
        worst = max(worst, err / den)
        worst_plain = max(worst_plain, np.linalg.norm(got[:3] - fd_h[:3]) / den)
        assert abs(got[3] - rich2[3]) <= 1e-3 * max(abs(rich2[3]), floor_a)
    print(f"position gradient vs FP64: analytic max {rel_p.max():.2e}, Richardson FD max {worst:.2e}, "
          f"plain central difference (h=1e-4) max {worst_plain:.2e}")
