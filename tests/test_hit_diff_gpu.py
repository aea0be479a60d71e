"""GPU checks of the differentiable hit query (rdn_hit_diff_forward /
rdn_hit_diff_adjoint) through the C ABI, wrapped in a test-only
torch.autograd.Function: the hit distance t, the barycentrics u, v and the
interpolated vertex attribute of the closest hit, and the gradients of any
function of them with respect to vertex positions, vertex attributes, ray
origins and ray directions, at frozen visibility.

The values differentiated are those of the reference's closest-hit query
(geometry/mod.rs:105-155, traverse_cpu.rs:157): t is the parameter along the
ray's direction as given. Checks: forward values against FP64 on the hit
triangle; every gradient against an FP64 analytic gradient (the same
frozen-visibility derivative in double) and against FP64 central differences
(h = 1e-4 on positions, origins and directions, Richardson-extrapolated);
instanced scenes with rotated, scaled and mirrored instances and non-unit ray
directions (world-space ray gradients)."""

import ctypes as C

import numpy as np
import pytest
import torch

from helpers import mat4_cols, orc, rot_x, rot_z, rt, scenes, single_mesh_scene, Scene
from rendiation_gb300 import native

pytestmark = pytest.mark.gpu


class HitQuery(torch.autograd.Function):
    """(origins, directions, positions, attributes) -> per-ray (t, u, v, value).
    Positions enter through the acceleration structure already built in
    `system`: the forward ignores the tensor's value, the backward returns its
    gradient."""

    @staticmethod
    def forward(ctx, origins, directions, positions, attributes, system, record=False, traversal=0):
        L = native.lib()
        n = origins.shape[0]
        rays = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
        rays[:, 0:3] = origins
        rays[:, 4:7] = directions
        rays[:, 7] = float("inf")
        hit = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        tri = torch.zeros(n, dtype=torch.int32, device="cuda")
        inst = torch.zeros(n, dtype=torch.int32, device="cuda")
        d = native.HitDiffDesc(rays.data_ptr(), n, 0, attributes.data_ptr(), hit.data_ptr(), tri.data_ptr(),
                               inst.data_ptr(), None, None, None, None, traversal, 0, 0, 0, 0)
        st = L.rdn_hit_diff_forward(system._h, C.byref(d), C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, L.rdn_last_error(system._h).decode()
        ctx.save_for_backward(rays, attributes, tri, inst)
        ctx.system, ctx.nv, ctx.record, ctx.traversal = system, positions.shape[0], record, traversal
        return hit

    @staticmethod
    def backward(ctx, g_hit):
        rays, attributes, tri, inst = ctx.saved_tensors
        L = native.lib()
        n = rays.shape[0]
        g_hit = g_hit.contiguous()
        gv = torch.zeros((ctx.nv, 4), dtype=torch.float32, device="cuda")
        go = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
        gd = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
        d = native.HitDiffDesc(rays.data_ptr(), n, 0, attributes.data_ptr(), None, tri.data_ptr(), inst.data_ptr(),
                               g_hit.data_ptr(), gv.data_ptr(), go.data_ptr(), gd.data_ptr(), ctx.traversal, 0,
                               int(ctx.record), 0, 0)
        st = L.rdn_hit_diff_adjoint(ctx.system._h, C.byref(d), C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, L.rdn_last_error(ctx.system._h).decode()
        return go, gd, gv[:, :3].contiguous(), gv[:, 3].contiguous(), None, None, None


def upstream(hit, w):
    """The test's scalar function of the hit query: linear and quadratic terms
    in every output, with per-ray weights w (n, 4)."""
    t, u, v, val = hit[:, 0], hit[:, 1], hit[:, 2], hit[:, 3]
    return (w[:, 0] * t + w[:, 1] * u + w[:, 2] * v + w[:, 3] * val + 0.5 * (u * u + t * t) + v * val).sum()


def solve64(o_w, d_w, tinv, v):
    """FP64 hit of world rays on frozen object-space triangles v (n, 3, 3):
    the object ray (affine inverse transform), then M (s, u, v) = o - v0 with
    M = [-d | e1 | e2]; returns s, u, v."""
    A = tinv.reshape(4, 4).T.astype(np.float64)  # column-major Mat4 -> row-major matrix
    o = o_w @ A[:3, :3].T + A[:3, 3]
    d = d_w @ A[:3, :3].T
    e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
    M = np.stack([-d, e1, e2], axis=2)
    x = np.linalg.solve(M, (o - v[:, 0])[..., None])[..., 0]
    return x[:, 0], x[:, 1], x[:, 2]


def object_ray_f32(o_w, d_w, tinv):
    """The object-space ray as the kernels form it in f32 (transform_inv times
    (o, 1), divided by w; the 3x3 part times d), one rounding per operation."""
    m = np.asarray(tinv, np.float32)
    o = np.asarray(o_w, np.float32)
    d = np.asarray(d_w, np.float32)
    f = np.float32

    def row(v, r, w):
        acc = (v[:, 0] * m[r]).astype(f)
        acc = (acc + (v[:, 1] * m[4 + r]).astype(f)).astype(f)
        acc = (acc + (v[:, 2] * m[8 + r]).astype(f)).astype(f)
        return (acc + (f(w) * m[12 + r]).astype(f)).astype(f) if w else acc

    ow = row(o, 3, 1)
    oo = np.stack([(row(o, r, 1) / ow).astype(f) for r in range(3)], 1)
    dd = np.stack([row(d, r, 0) for r in range(3)], 1)
    return oo.astype(np.float64), dd.astype(np.float64)


def loss64(o_w, d_w, pos, attr, idx, tri, tinv, w):
    tv = idx.reshape(-1, 3)[tri]
    s, u, v = solve64(o_w, d_w, tinv, pos[tv])
    val = (1 - u - v) * attr[tv[:, 0]] + u * attr[tv[:, 1]] + v * attr[tv[:, 2]]
    hit = np.stack([s, u, v, val], 1)
    return float(upstream(hit, w))


def run_case(P, mesh, tinv, origins, dirs, attr, traversal=0, record=False, seed=3, fd_samples=48):
    rng = np.random.default_rng(seed)
    n = origins.shape[0]
    d_o = torch.from_numpy(origins.astype(np.float32)).cuda().requires_grad_(True)
    d_d = torch.from_numpy(dirs.astype(np.float32)).cuda().requires_grad_(True)
    d_p = torch.from_numpy(mesh.positions.copy()).cuda().requires_grad_(True)
    d_a = torch.from_numpy(attr).cuda().requires_grad_(True)
    hit = HitQuery.apply(d_o, d_d, d_p, d_a, P, record, traversal)
    tri = None
    w = rng.normal(size=(n, 4))
    L = upstream(hit.double(), torch.from_numpy(w).cuda())
    L.backward()
    h = hit.detach().cpu().numpy().astype(np.float64)
    g_o, g_d = d_o.grad.cpu().numpy(), d_d.grad.cpu().numpy()
    g_p, g_a = d_p.grad.cpu().numpy(), d_a.grad.cpu().numpy()
    # which triangle each ray hit: re-run the forward for the records
    L_ = native.lib()
    rays = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
    rays[:, 0:3] = d_o.detach()
    rays[:, 4:7] = d_d.detach()
    rays[:, 7] = float("inf")
    t_tri = torch.zeros(n, dtype=torch.int32, device="cuda")
    dd = native.HitDiffDesc(rays.data_ptr(), n, 0, d_a.data_ptr(), None, t_tri.data_ptr(), None, None, None, None,
                            None, traversal, 0, 0, 0, 0)
    assert L_.rdn_hit_diff_forward(P._h, C.byref(dd), None) == 0
    tri = t_tri.cpu().numpy().view(np.uint32)
    hitm = tri != orc.MISS
    assert hitm.mean() > 0.5
    # the built triangle index equals the mesh's own (one geometry)
    idx = mesh.indices.reshape(-1, 3) if mesh.indices is not None else np.arange(mesh.positions.shape[0]).reshape(-1, 3)
    pos = mesh.positions.astype(np.float64)
    a64 = attr.astype(np.float64)
    o64, d64 = origins.astype(np.float32).astype(np.float64), dirs.astype(np.float32).astype(np.float64)
    # FP64 references are taken on the f32 object-space ray that the kernels form
    # (an f32 step of the reference's own traversal, traverse_cpu.rs:99-104);
    # world-space ray gradients follow by the chain rule: g_world = g_object @ A3
    oo, do = object_ray_f32(o64, d64, tinv)
    A3 = np.asarray(tinv, np.float64).reshape(4, 4).T[:3, :3]
    ident = np.eye(4).reshape(-1)
    sel = np.nonzero(hitm)[0]
    tv = idx[tri[sel]]
    s, u, v = solve64(oo[sel], do[sel], ident, pos[tv])
    val = (1 - u - v) * a64[tv[:, 0]] + u * a64[tv[:, 1]] + v * a64[tv[:, 2]]
    assert np.max(np.abs(h[sel, 0] - s) / np.abs(s)) < 2e-6
    assert np.max(np.abs(h[sel, 1] - u)) < 2e-6 and np.max(np.abs(h[sel, 2] - v)) < 2e-6
    assert np.max(np.abs(h[sel, 3] - val)) < 4e-6
    assert np.all(h[~hitm, 1:] == 0)
    # FP64 analytic gradient: G = dL/d(t, u, v, value) at the FP64 outputs
    ws = w[sel]
    G = np.stack([ws[:, 0] + s, ws[:, 1] + u, ws[:, 2] + val, ws[:, 3] + v], 1)
    gu = G[:, 1] + G[:, 3] * (a64[tv[:, 1]] - a64[tv[:, 0]])
    gv = G[:, 2] + G[:, 3] * (a64[tv[:, 2]] - a64[tv[:, 0]])
    e1, e2 = pos[tv[:, 1]] - pos[tv[:, 0]], pos[tv[:, 2]] - pos[tv[:, 0]]
    M = np.stack([-do[sel], e1, e2], axis=2)
    lam = np.linalg.solve(np.transpose(M, (0, 2, 1)), np.stack([G[:, 0], gu, gv], 1)[..., None])[..., 0]
    ga, gp = np.zeros(a64.shape[0]), np.zeros((a64.shape[0], 3))
    for k, wk in enumerate([1 - u - v, u, v]):
        np.add.at(ga, tv[:, k], G[:, 3] * wk)
        np.add.at(gp, tv[:, k], -wk[:, None] * lam)
    go64 = lam @ A3
    gd64 = s[:, None] * go64

    def rel(got, ref):
        nrm = np.linalg.norm(ref, axis=-1) if ref.ndim > 1 else np.abs(ref)
        floor = 1e-2 * np.median(nrm[nrm > 0])
        diff = np.linalg.norm(got - ref, axis=-1) if ref.ndim > 1 else np.abs(got - ref)
        return diff / np.maximum(nrm, floor)

    errs = {"positions": rel(g_p, gp).max(), "attributes": rel(g_a, ga).max(),
            "origins": rel(g_o[sel], go64).max(), "directions": rel(g_d[sel], gd64).max()}
    for k, e in errs.items():
        assert e < 1e-3, (k, errs)
    assert np.all(g_o[~hitm] == 0) and np.all(g_d[~hitm] == 0)

    # FP64 central differences (frozen triangles) in object space, Richardson-extrapolated from h and h/2
    def fd(fun, x0, hh):
        return (fun(x0 + hh) - fun(x0 - hh)) / (2 * hh)

    def rich(fun, x0, hh=1e-4):
        return (4 * fd(fun, x0, hh / 2) - fd(fun, x0, hh)) / 3

    pick_r = rng.choice(sel, size=min(fd_samples, sel.size), replace=False)
    for i in pick_r:
        f_o, f_d = np.zeros(3), np.zeros(3)
        for c in range(3):
            def fo(x, i=i, c=c):
                o2 = oo[[i]].copy()
                o2[0, c] = x
                return loss64(o2, do[[i]], pos, a64, idx, tri[[i]], ident, w[[i]])

            def fdd(x, i=i, c=c):
                d2 = do[[i]].copy()
                d2[0, c] = x
                return loss64(oo[[i]], d2, pos, a64, idx, tri[[i]], ident, w[[i]])

            f_o[c], f_d[c] = rich(fo, oo[i, c]), rich(fdd, do[i, c])
        ref_o, ref_d = f_o @ A3, f_d @ A3
        k = np.nonzero(sel == i)[0][0]
        den_o, den_d = max(np.linalg.norm(go64[k]), 1e-6), max(np.linalg.norm(gd64[k]), 1e-6)
        assert np.linalg.norm(g_o[i] - ref_o) <= 1e-3 * den_o, ("origin", i, g_o[i], ref_o)
        assert np.linalg.norm(g_d[i] - ref_d) <= 1e-3 * den_d, ("direction", i, g_d[i], ref_d)
    seen = np.unique(tv.reshape(-1))
    pick_v = rng.choice(seen, size=min(fd_samples, seen.size), replace=False)
    for vi in pick_v:
        rows = np.nonzero(np.any(tv == vi, axis=1))[0]
        rsel = sel[rows]
        for c in range(4):
            def f_v(x, vi=vi, c=c):
                p2, a2 = pos.copy(), a64.copy()
                if c < 3:
                    p2[vi, c] = x
                else:
                    a2[vi] = x
                return loss64(oo[rsel], do[rsel], p2, a2, idx, tri[rsel], ident, w[rsel])

            x0 = pos[vi, c] if c < 3 else a64[vi]
            ref = rich(f_v, x0)
            got = g_p[vi, c] if c < 3 else g_a[vi]
            den = max(np.linalg.norm(gp[vi]) if c < 3 else abs(ga[vi]), 1e-2 * np.median(np.abs(ga[ga != 0])))
            assert abs(got - ref) <= 1e-3 * den, ("vertex", vi, c, got, ref)
    return errs


@pytest.fixture(scope="module")
def field():
    mesh = scenes.heightfield(64, seed=3)
    attr = np.random.default_rng(5).random(mesh.positions.shape[0]).astype(np.float32)
    sc = single_mesh_scene(mesh)
    return mesh, attr, sc.build_product()


@pytest.mark.parametrize("record", [False, True])
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED_WIDE])
def test_gradients_identity_instance(field, record, traversal, cuda):
    mesh, attr, P = field
    cam = scenes.PinholeCamera.look_at((0.5, -0.2, 0.9), (0.5, 0.5, 0.0), 35.0, 64, 64)
    rays = scenes.pinhole_rays(cam)
    run_case(P, mesh, np.eye(4, dtype=np.float32).reshape(-1), rays["org"], rays["dir"], attr, traversal, record)


def test_gradients_non_unit_directions(field, cuda):
    """Directions scaled by 0.3..3: t is the parameter along the given
    direction, and its gradient follows."""
    mesh, attr, P = field
    cam = scenes.PinholeCamera.look_at((0.5, -0.2, 0.9), (0.5, 0.5, 0.0), 35.0, 48, 48)
    rays = scenes.pinhole_rays(cam)
    k = np.random.default_rng(1).uniform(0.3, 3.0, rays.shape[0]).astype(np.float32)
    run_case(P, mesh, np.eye(4, dtype=np.float32).reshape(-1), rays["org"], rays["dir"] * k[:, None], attr)


@pytest.mark.parametrize("xf", [0, 1])
def test_gradients_through_an_instance_transform(xf, cuda):
    """One instance with a rotation, a non-uniform (and, for xf 1, mirrored)
    scale and a translation: vertex gradients in object space, ray gradients
    in world space."""
    mesh = scenes.heightfield(48, seed=4)
    attr = np.random.default_rng(6).random(mesh.positions.shape[0]).astype(np.float32)
    m = (mat4_cols(rot_z(0.6) @ rot_x(0.2), (1.3, 0.8, 1.1), (0.2, -0.1, 0.05)) if xf == 0
         else mat4_cols(rot_z(-0.9), (-1.0, 1.2, 0.9), (0.9, 0.3, -0.1)))
    sc = Scene([[(mesh.positions, mesh.indices, 1)]], [[{"blas": 0, "transform": m}]])
    P = sc.build_product()
    # the instance's f32 inverse transform as built (DeviceInstance: transform[16], transform_inv[16], ...)
    tinv = np.frombuffer(P.built_array("tlas_data"), np.float32)[16:32].astype(np.float64)
    centre = m.reshape(4, 4).T.astype(np.float64) @ np.array([0.5, 0.5, 0.0, 1.0])
    cam = scenes.PinholeCamera.look_at(tuple(centre[:3] + np.array([0.1, -0.9, 1.2])), tuple(centre[:3]), 40.0, 48, 48)
    rays = scenes.pinhole_rays(cam)
    run_case(P, mesh, tinv, rays["org"], rays["dir"], attr)


def test_errors_and_misses(field, cuda):
    mesh, attr, P = field
    L = native.lib()
    d = native.HitDiffDesc()
    d.count = 4
    assert L.rdn_hit_diff_forward(P._h, C.byref(d), None) == -1  # null rays
    rays = torch.zeros((4, 8), device="cuda")
    rays[:, 2] = 5.0
    rays[:, 6] = 1.0  # pointing away from the field: all miss
    rays[:, 7] = 7.0
    hit = torch.full((4, 4), -1.0, device="cuda")
    d.rays, d.hit = rays.data_ptr(), hit.data_ptr()
    assert L.rdn_hit_diff_adjoint(P._h, C.byref(d), None) == -1  # adjoint without gradients
    assert L.rdn_hit_diff_forward(P._h, C.byref(d), None) == 0
    torch.cuda.synchronize()
    assert hit.cpu().numpy().tolist() == [[7.0, 0.0, 0.0, 0.0]] * 4
