"""Differentiable paths (rdn_attr_paths_*) through instanced scenes: heightfields
placed by random rotations, scales (some negative, mirroring the instance) and
translations, several instances of one BLAS. The benchmark configurations use
identity instances only; here the segment rays and hit triangles must still
equal the oracle's, and values and vertex gradients (accumulated over every
instance of a vertex, in the BLAS's object space) must agree with an FP64
evaluation on the object-space rays the kernels form."""

import ctypes as C

import numpy as np
import pytest
import torch

from helpers import Scene, orc, rt, scenes
from rendiation_gb300 import native
from test_adjoint_paths_gpu import SEG, desc, fp64_bary
from test_fuzz_gpu import random_rotation

pytestmark = pytest.mark.gpu
F = np.float32


def object_rays(seg_rays, inv):
    """The object-space ray the adjoint kernels re-solve on, in FP32: the origin as to_instance
    forms it (transform_inv * (o, 1) / w) and the direction to_mat3(transform_inv) * d before
    normalisation (Cramer's rule does not depend on its length, and normalising would round
    it once more). rays (n,) x inv (n, 16)."""
    o = np.stack([seg_rays["org"][:, k] for k in range(3)], 1).astype(F)
    d = np.stack([seg_rays["dir"][:, k] for k in range(3)], 1).astype(F)

    def row(v, w, k):
        acc = (v[:, 0] * inv[:, k]).astype(F) + (v[:, 1] * inv[:, 4 + k]).astype(F)
        acc = acc.astype(F) + (v[:, 2] * inv[:, 8 + k]).astype(F)
        return (acc.astype(F) + (w * inv[:, 12 + k]).astype(F)).astype(F) if w is not None else acc.astype(F)

    one = np.ones(o.shape[0], F)
    x, y, z, w = (row(o, one, k) for k in range(4))
    bo = np.stack([x / w, y / w, z / w], 1).astype(F)
    bd = np.stack([row(d, None, k) for k in range(3)], 1).astype(F)
    out = np.zeros(seg_rays.shape[0], seg_rays.dtype)
    out["org"], out["dir"] = bo, bd
    return out


def instanced_scene(seed):
    rng = np.random.default_rng(500 + seed)
    meshes = [scenes.heightfield(int(n), seed=30 + seed * 7 + k) for k, n in enumerate(rng.integers(6, 20, 3))]
    inst = []
    for k in range(6):
        m = np.eye(4)
        s = rng.uniform(0.6, 1.4, 3) * rng.choice([-1.0, 1.0], 3, p=[0.25, 0.75])
        m[:3, :3] = random_rotation(rng) @ np.diag(s)
        m[:3, 3] = rng.uniform(-0.8, 0.8, 3)
        inst.append({"blas": k % len(meshes), "transform": m.T.reshape(-1).astype(F)})
    sc = Scene([[(m.positions, m.indices, 1)] for m in meshes], [inst])
    pos = np.concatenate([m.positions for m in meshes])
    offs = np.cumsum([0] + [m.positions.shape[0] for m in meshes])
    idx = np.concatenate([m.indices + offs[k] for k, m in enumerate(meshes)]).astype(np.uint32)
    rays = scenes.sphere_rays(40000, (-1.2, -1.2, -1.2), (1.2, 1.2, 1.2), seed=900 + seed)
    return sc, pos, idx, rays, rng


@pytest.mark.parametrize("seed", range(4))
def test_instanced_attr_paths(seed, cuda):
    sc, pos, idx, rays, rng = instanced_scene(seed)
    S, P = sc.build_oracle(), sc.build_product()
    L = native.lib()
    n = rays.shape[0]
    tidx = np.zeros(n, np.uint32)
    attr = rng.random(pos.shape[0]).astype(F)
    targets = rng.random(n * SEG).astype(F)
    d_rays = torch.from_numpy(rays.view(F).reshape(-1, 8).copy()).cuda()
    d_tidx = torch.from_numpy(tidx.astype(np.int32)).cuda()
    d_attr = torch.from_numpy(attr).cuda()
    d_tgt = torch.from_numpy(targets).cuda()
    values = torch.zeros(n * SEG, device="cuda")
    seg_tri = torch.zeros(n * SEG, dtype=torch.int32, device="cuda")
    seg_inst = torch.zeros(n * SEG, dtype=torch.int32, device="cuda")
    seg_rays = torch.zeros((n * SEG, 8), device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = torch.zeros((pos.shape[0], 4), device="cuda")
    fwd = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), values=values.data_ptr(),
               loss_sum=loss.data_ptr(), seg_tri=seg_tri.data_ptr(), seg_rays=seg_rays.data_ptr(),
               seg_inst=seg_inst.data_ptr(), traversal=rt.TRAVERSAL_REFERENCE)
    adj = desc(d_rays, d_tidx, n, d_attr, targets=d_tgt.data_ptr(), grad_vertices=grad.data_ptr(),
               traversal=rt.TRAVERSAL_REFERENCE)
    assert L.rdn_attr_paths_forward(P._h, C.byref(fwd), None) == 0
    assert L.rdn_attr_paths_adjoint(P._h, C.byref(adj), None) == 0
    torch.cuda.synchronize()

    exp_rays, exp_tri = orc.path_segments(S, rays, tidx, segments=SEG, seed=9, threads=8)
    got_tri = seg_tri.cpu().numpy().view(np.uint32)
    assert np.array_equal(got_tri, exp_tri)
    alive = exp_tri != orc.MISS
    assert alive.sum() > 500
    got_rays = seg_rays.cpu().numpy().view(exp_rays.dtype).reshape(-1)
    assert np.array_equal(got_rays[alive].view(np.uint32), exp_rays[alive].view(np.uint32))

    # FP64 on the FP32 object-space rays of the hit instances
    tdata = np.frombuffer(S.buffer(3), np.uint8).reshape(-1, 144)
    inv_all = tdata[:, 64:128].copy().view(F)
    inst = seg_inst.cpu().numpy().view(np.uint32)[alive]
    sr, tri = object_rays(exp_rays[alive], inv_all[inst]), exp_tri[alive]
    u, v, M = fp64_bary(pos, idx, sr, tri)
    tv = idx.reshape(-1, 3)[tri]
    a = attr.astype(np.float64)
    val = (1 - u - v) * a[tv[:, 0]] + u * a[tv[:, 1]] + v * a[tv[:, 2]]
    got_val = values.cpu().numpy()
    assert np.max(np.abs(got_val[alive] - val)) < 2e-6
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
