"""GPU checks of the batched differentiable paths (rdn_attr_paths_*): several
heightfields of different size in one launch, 3 segments per path (primary +
2 diffuse bounces). Segment rays and hit triangles equal the oracle's; values,
loss and gradients agree with an FP64 evaluation on the same segments; the
captured forward+adjoint graph reproduces the separate calls."""

import ctypes as C

import numpy as np
import pytest
import torch

from helpers import Scene, orc, rt, scenes
from rendiation_gb300 import native

pytestmark = pytest.mark.gpu
SEG = 3


def fp64_bary(pos, idx, seg_rays, tri):
    v = pos.astype(np.float64)[idx.reshape(-1, 3)[tri]]
    o = seg_rays["org"].astype(np.float64)
    d = seg_rays["dir"].astype(np.float64)
    e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    M = np.stack([-d, e1, e2], axis=2)
    x = np.linalg.solve(M, (o - v[:, 0])[..., None])[..., 0]
    dhat = d / np.linalg.norm(d, axis=1, keepdims=True)
    return x[:, 1], x[:, 2], np.stack([-dhat, e1, e2], axis=2)


@pytest.fixture(scope="module")
def fields():
    meshes = [scenes.heightfield(n, seed=10 + k) for k, n in enumerate((24, 40, 64, 33))]
    sc = Scene([[(m.positions, m.indices, 1)] for m in meshes], [[{"blas": s}] for s in range(len(meshes))])
    rays, tidx = [], []
    for s in range(len(meshes)):
        cam = scenes.PinholeCamera.look_at((0.5, -0.4, 0.9), (0.5, 0.5, 0.0), 30.0, 40 + 8 * s, 32)
        r = scenes.pinhole_rays(cam)
        rays.append(r)
        tidx.append(np.full(r.shape[0], s, np.uint32))
    rays = np.concatenate(rays)
    tidx = np.concatenate(tidx)
    pos = np.concatenate([m.positions for m in meshes])
    offs = np.cumsum([0] + [m.positions.shape[0] for m in meshes])
    idx = np.concatenate([m.indices + offs[k] for k, m in enumerate(meshes)]).astype(np.uint32)
    attr = np.random.default_rng(2).random(pos.shape[0]).astype(np.float32)
    return sc.build_oracle(), sc.build_product(), rays, tidx, pos, idx, attr


def desc(d_rays, d_tidx, n, d_attr, **kw):
    d = native.AttrPathDesc()
    d.rays, d.tlas_idx, d.count, d.segments, d.seed = d_rays.data_ptr(), d_tidx.data_ptr(), n, SEG, 9
    d.attributes = d_attr.data_ptr()
    d.grad_scale = 1.0
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_paths_forward_adjoint(fields, cuda):
    S, P, rays, tidx, pos, idx, attr = fields
    L = native.lib()
    n = rays.shape[0]
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_tidx = torch.from_numpy(tidx.astype(np.int32)).cuda()
    d_attr = torch.from_numpy(attr).cuda()
    rng = np.random.default_rng(4)
    targets = rng.random(n * SEG).astype(np.float32)
    d_tgt = torch.from_numpy(targets).cuda()
    values = torch.zeros(n * SEG, device="cuda")
    seg_tri = torch.zeros(n * SEG, dtype=torch.int32, device="cuda")
    seg_rays = torch.zeros((n * SEG, 8), device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = torch.zeros((pos.shape[0], 4), device="cuda")
    fwd = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), values=values.data_ptr(),
               loss_sum=loss.data_ptr(), seg_tri=seg_tri.data_ptr(), seg_rays=seg_rays.data_ptr(),
               traversal=rt.TRAVERSAL_REFERENCE)
    adj = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), grad_vertices=grad.data_ptr(),
               traversal=rt.TRAVERSAL_REFERENCE)
    assert L.rdn_attr_paths_forward(P._h, C.byref(fwd), None) == 0
    assert L.rdn_attr_paths_adjoint(P._h, C.byref(adj), None) == 0
    torch.cuda.synchronize()

    exp_rays, exp_tri = orc.path_segments(S, rays, tidx, segments=SEG, seed=9, threads=4)
    got_tri = seg_tri.cpu().numpy().view(np.uint32)
    assert np.array_equal(got_tri, exp_tri)
    alive = exp_tri != orc.MISS
    assert alive.reshape(-1, SEG)[:, 2].sum() > 50  # some paths reach the second bounce
    got_rays = seg_rays.cpu().numpy().view(exp_rays.dtype).reshape(-1)
    assert np.array_equal(got_rays[alive].view(np.uint32), exp_rays[alive].view(np.uint32))

    # FP64 values, loss and gradients on the same segments
    sr, tri = exp_rays[alive], exp_tri[alive]
    u, v, M = fp64_bary(pos, idx, sr, tri)
    tv = idx.reshape(-1, 3)[tri]
    a = attr.astype(np.float64)
    val = (1 - u - v) * a[tv[:, 0]] + u * a[tv[:, 1]] + v * a[tv[:, 2]]
    got_val = values.cpu().numpy()
    assert np.max(np.abs(got_val[alive] - val)) < 2e-6
    assert np.all(got_val[~alive] == 0)
    t64 = targets.astype(np.float64)
    loss64 = np.sum((val - t64[alive]) ** 2) + np.sum(t64[~alive] ** 2)
    assert abs(loss.item() - loss64) < 1e-5 * loss64
    r = 2 * (val - t64[alive])
    g = np.stack([np.zeros_like(r), r * (a[tv[:, 1]] - a[tv[:, 0]]), r * (a[tv[:, 2]] - a[tv[:, 0]])], 1)
    lam = np.linalg.solve(np.transpose(M, (0, 2, 1)), g[..., None])[..., 0]
    gp = np.zeros((a.shape[0], 3))
    ga = np.zeros(a.shape[0])
    for k, wk in enumerate([1 - u - v, u, v]):
        np.add.at(gp, tv[:, k], -wk[:, None] * lam)
        np.add.at(ga, tv[:, k], r * wk)
    gg = grad.cpu().numpy().astype(np.float64)
    norm = np.linalg.norm(gp, axis=1)
    rel = np.linalg.norm(gg[:, :3] - gp, axis=1) / np.maximum(norm, 1e-2 * np.median(norm[norm > 0]))
    rela = np.abs(gg[:, 3] - ga) / np.maximum(np.abs(ga), 1e-2 * np.median(np.abs(ga[ga != 0])))
    assert rel.max() < 1e-3, rel.max()
    assert rela.max() < 1e-3, rela.max()

    # one captured graph for forward + adjoint reproduces the separate calls
    g_handle = C.c_void_p()
    both = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), loss_sum=loss.data_ptr(),
                grad_vertices=grad.data_ptr(), traversal=rt.TRAVERSAL_ORDERED)
    assert L.rdn_attr_paths_graph(P._h, C.byref(both), pos.shape[0], C.byref(g_handle)) == 0
    for _ in range(2):
        assert L.rdn_graph_launch(g_handle, None) == 0
    torch.cuda.synchronize()
    L.rdn_graph_destroy(g_handle)
    gg2 = grad.cpu().numpy().astype(np.float64)
    rel2 = np.linalg.norm(gg2[:, :3] - gp, axis=1) / np.maximum(norm, 1e-2 * np.median(norm[norm > 0]))
    assert rel2.max() < 1e-3
    assert abs(loss.item() - loss64) < 1e-5 * loss64


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE])
def test_paths_adjoint_from_record(fields, traversal, cuda):
    """The adjoint that differentiates the forward's recorded segments (seg_tri,
    seg_inst, seg_rays) equals the adjoint that traces the paths again, and
    the FP64 gradient of exactly the recorded segments; so does the captured
    forward + recorded-adjoint graph."""
    S, P, rays, tidx, pos, idx, attr = fields
    L = native.lib()
    n = rays.shape[0]
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_tidx = torch.from_numpy(tidx.astype(np.int32)).cuda()
    d_attr = torch.from_numpy(attr).cuda()
    targets = np.random.default_rng(5).random(n * SEG).astype(np.float32)
    d_tgt = torch.from_numpy(targets).cuda()
    seg_tri = torch.zeros(n * SEG, dtype=torch.int32, device="cuda")
    seg_inst = torch.zeros(n * SEG, dtype=torch.int32, device="cuda")
    seg_rays = torch.zeros((n * SEG, 8), device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    g_rec = torch.zeros((pos.shape[0], 4), device="cuda")
    g_trace = torch.zeros((pos.shape[0], 4), device="cuda")
    rec = dict(seg_tri=seg_tri.data_ptr(), seg_inst=seg_inst.data_ptr(), seg_rays=seg_rays.data_ptr())
    fwd = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), loss_sum=loss.data_ptr(), traversal=traversal,
               **rec)
    assert L.rdn_attr_paths_forward(P._h, C.byref(fwd), None) == 0
    adj_rec = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), grad_vertices=g_rec.data_ptr(),
                   traversal=traversal, from_record=1, **rec)
    assert L.rdn_attr_paths_adjoint(P._h, C.byref(adj_rec), None) == 0
    adj_tr = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), grad_vertices=g_trace.data_ptr(),
                  traversal=rt.TRAVERSAL_REFERENCE)
    assert L.rdn_attr_paths_adjoint(P._h, C.byref(adj_tr), None) == 0
    torch.cuda.synchronize()
    inst = seg_inst.cpu().numpy().view(np.uint32)
    tri = seg_tri.cpu().numpy().view(np.uint32)
    alive = tri != orc.MISS
    assert np.all(inst[~alive] == orc.MISS) and np.all(inst[alive] < len(tidx))
    assert np.array_equal(inst.reshape(-1, SEG)[alive.reshape(-1, SEG)[:, 0], 0],
                          tidx[alive.reshape(-1, SEG)[:, 0]])  # identity instances: slot = scene

    # FP64 gradient of the recorded segments
    sr = seg_rays.cpu().numpy().view(scenes.RAY_DTYPE).reshape(-1)[alive]
    u, v, M = fp64_bary(pos, idx, sr, tri[alive])
    tv = idx.reshape(-1, 3)[tri[alive]]
    a = attr.astype(np.float64)
    val = (1 - u - v) * a[tv[:, 0]] + u * a[tv[:, 1]] + v * a[tv[:, 2]]
    r = 2 * (val - targets.astype(np.float64)[alive])
    g = np.stack([np.zeros_like(r), r * (a[tv[:, 1]] - a[tv[:, 0]]), r * (a[tv[:, 2]] - a[tv[:, 0]])], 1)
    lam = np.linalg.solve(np.transpose(M, (0, 2, 1)), g[..., None])[..., 0]
    gp = np.zeros((a.shape[0], 3))
    for k, wk in enumerate([1 - u - v, u, v]):
        np.add.at(gp, tv[:, k], -wk[:, None] * lam)
    norm = np.linalg.norm(gp, axis=1)
    floor = 1e-2 * np.median(norm[norm > 0])
    gr = g_rec.cpu().numpy().astype(np.float64)
    assert (np.linalg.norm(gr[:, :3] - gp, axis=1) / np.maximum(norm, floor)).max() < 1e-4
    if traversal == rt.TRAVERSAL_REFERENCE:  # same hits as the re-traced adjoint: only the atomic order differs
        gt = g_trace.cpu().numpy().astype(np.float64)
        assert (np.linalg.norm(gr - gt, axis=1) / np.maximum(np.linalg.norm(gt, axis=1), floor)).max() < 1e-5

    # the captured graph: forward (recording) + adjoint from the record
    g_handle = C.c_void_p()
    g_rec.zero_()
    both = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), loss_sum=loss.data_ptr(),
                grad_vertices=g_rec.data_ptr(), traversal=traversal, from_record=1, **rec)
    assert L.rdn_attr_paths_graph(P._h, C.byref(both), pos.shape[0], C.byref(g_handle)) == 0
    for _ in range(2):
        assert L.rdn_graph_launch(g_handle, None) == 0
    torch.cuda.synchronize()
    L.rdn_graph_destroy(g_handle)
    gr2 = g_rec.cpu().numpy().astype(np.float64)
    assert np.array_equal(seg_tri.cpu().numpy().view(np.uint32), tri)
    assert (np.linalg.norm(gr2[:, :3] - gp, axis=1) / np.maximum(norm, floor)).max() < 1e-4


def test_adjoint_from_record_needs_the_record(fields, cuda):
    S, P, rays, tidx, pos, idx, attr = fields
    L = native.lib()
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_tidx = torch.from_numpy(tidx.astype(np.int32)).cuda()
    d_attr = torch.from_numpy(attr).cuda()
    grad = torch.zeros((pos.shape[0], 4), device="cuda")
    adj = desc(d_rays, d_tidx, rays.shape[0], d_attr, grad_vertices=grad.data_ptr(), from_record=1)
    assert L.rdn_attr_paths_adjoint(P._h, C.byref(adj), None) == -1  # RDN_ERR_INVALID_ARG
