"""Seeded random scenes against the oracle: many small BLAS of different kinds
(soups, heightfields, axis-aligned cube stacks with coplanar faces and shared
edges, soups with zero-area triangles, indexed and non-indexed, opaque and
non-opaque geometries), TLAS with random rotations, scales (negative ones
mirror the instance), masks, instance flags and deleted slots, and rays that
include axis-parallel directions, origins on cube faces and finite ranges,
under random ray flags, cull masks and any-hit policies.

The GPU build must give the host build's arrays and the same four-child traces.
Reference order must equal the oracle bit for bit (NaN compared as NaN). The
ordered walks must agree on hit / miss for every ray, and on the hit itself
except exact-distance ties and rays that can meet a NaN distance (the oracle's
nan_exposure: a zero-area triangle, or a ray lying in a triangle's plane, whose
NaN makes the reference's own result depend on its walk order)."""

import numpy as np
import pytest
import torch

import naive_fixture as nf
from helpers import Scene, orc, rt, scenes
from test_trace_gpu import ORDERED_MODES, run_product

pytestmark = pytest.mark.gpu

SEEDS = range(16)


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def transform(rng):
    """Mat4 in the reference's column order; some identity, some axis-aligned
    integer placements (exact), some general."""
    kind = rng.integers(0, 3)
    m = np.eye(4)
    if kind == 1:
        m[:3, 3] = rng.integers(-2, 3, 3)
    elif kind == 2:
        s = rng.uniform(0.5, 1.5, 3) * rng.choice([-1.0, 1.0], 3, p=[0.2, 0.8])
        m[:3, :3] = random_rotation(rng) @ np.diag(s)
        m[:3, 3] = rng.uniform(-1.5, 1.5, 3)
    return m.T.reshape(-1).astype(np.float32)


def cube_stack(rng):
    """Unit cubes on integer positions: coplanar faces, shared edges, ties."""
    c = nf.cube()
    n = int(rng.integers(1, 6))
    pos = rng.integers(-1, 2, (n, 3)).astype(np.float32)
    p = np.concatenate([c.positions + q for q in pos])
    i = np.concatenate([c.indices + 24 * k for k in range(n)]).astype(np.uint32)
    return p, i


def degenerate_soup(rng):
    m = scenes.triangle_soup(int(rng.integers(50, 400)), seed=int(rng.integers(1 << 30)), offset=0.1)
    p = m.positions.reshape(-1, 3, 3).copy()
    k = rng.random(p.shape[0]) < 0.1
    p[k, 1] = p[k, 0]  # zero-area triangles
    return p.reshape(-1, 3), None


def geometry(rng):
    kind = rng.integers(0, 4)
    if kind == 0:
        m = scenes.triangle_soup(int(rng.integers(20, 1500)), seed=int(rng.integers(1 << 30)),
                                 offset=float(rng.uniform(0.01, 0.2)))
        p, i = m.positions, None
    elif kind == 1:
        m = scenes.heightfield(int(rng.integers(3, 20)), seed=int(rng.integers(1 << 30)))
        p, i = m.positions, m.indices
    elif kind == 2:
        p, i = cube_stack(rng)
    else:
        p, i = degenerate_soup(rng)
    flags = int(rng.random() < 0.8)  # opaque
    return (np.ascontiguousarray(p, np.float32), i, flags)


def random_scene(seed):
    rng = np.random.default_rng(1000 + seed)
    nb = int(rng.integers(1, 5))
    blas = [[geometry(rng) for _ in range(int(rng.integers(1, 3)))] for _ in range(nb)]
    deleted = [int(rng.integers(0, nb))] if nb > 1 and rng.random() < 0.3 else []
    live = [b for b in range(nb) if b not in deleted]
    tlas = []
    for _ in range(int(rng.integers(1, 4))):
        inst = []
        for _ in range(int(rng.integers(1, 7))):
            inst.append({"blas": int(rng.choice(live)), "transform": transform(rng),
                         "custom": int(rng.integers(0, 1 << 20)), "mask": int(rng.integers(1, 256)),
                         "flags": int(rng.integers(0, 16))})
        tlas.append(inst)
    return Scene(blas, tlas, deleted_blas=deleted, blas_bin_size=int(rng.choice([1, 2, 4]))), rng


def random_rays(rng, n):
    r = scenes.sphere_rays(n, (-1.5, -1.5, -1.5), (2.5, 2.5, 2.5), seed=int(rng.integers(1 << 30)))
    # axis-parallel directions from integer-grid and half-integer origins
    k = n // 4
    axes = np.eye(3, dtype=np.float32)[rng.integers(0, 3, k)] * rng.choice([-1.0, 1.0], (k, 1)).astype(np.float32)
    org = rng.integers(-2, 3, (k, 3)).astype(np.float32) + rng.choice([0.0, 0.5, 0.25], (k, 3)).astype(np.float32)
    r2 = scenes.make_rays(org, axes)
    rays = np.concatenate([r, r2])
    fin = rng.random(rays.shape[0]) < 0.2
    rays["tmax"][fin] = rng.uniform(0.1, 3.0, fin.sum()).astype(np.float32)
    late = rng.random(rays.shape[0]) < 0.1
    rays["tmin"][late] = rng.uniform(0.0, 1.0, late.sum()).astype(np.float32)
    return rays


FLAG_CHOICES = [0, rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES, rt.RAY_FLAG_CULL_FRONT_FACING_TRIANGLES,
                rt.RAY_FLAG_FORCE_OPAQUE, rt.RAY_FLAG_FORCE_NON_OPAQUE, rt.RAY_FLAG_CULL_OPAQUE,
                rt.RAY_FLAG_CULL_NON_OPAQUE, rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH,
                rt.RAY_FLAG_FORCE_NON_OPAQUE | rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES]


def same_bits_nan(a, b):
    nan = np.isnan(a)
    return np.array_equal(nan, np.isnan(b)) and np.array_equal(a[~nan].view(np.uint32), b[~nan].view(np.uint32))


@pytest.mark.parametrize("seed", SEEDS)
def test_random_scene(seed, cuda):
    sc, rng = random_scene(seed)
    try:
        S = sc.build_oracle()
    except RuntimeError as e:
        # a multi-geometry BLAS shifts the per-geometry root boxes of later BLAS slots
        # (naive/mod.rs:239, 272-275); a lookup that lands on a missing box panics in the
        # reference, and the product refuses the same scene
        assert "missing BLAS box" in str(e)
        with pytest.raises(RuntimeError):
            sc.build_product()
        with pytest.raises(RuntimeError):
            sc.build_product(device_build=True)
        return
    P = sc.build_product()
    # the GPU build of the same scene: the reference-layout arrays byte for byte
    D = sc.build_product(device_build=True)
    for name in rt.BUILT_ARRAYS:
        assert D.built_array(name) == P.built_array(name), (seed, name)
    rays = random_rays(rng, 12000)
    n_tlas = len(sc.tlas)
    tidx = rng.integers(0, n_tlas, rays.shape[0]).astype(np.uint32)
    for case in range(3):
        flags = int(rng.choice(FLAG_CHOICES))
        mask = int(rng.choice([0xFF, int(rng.integers(1, 256))]))
        anyhit = int(rng.integers(0, 3))
        expect, _ = S.trace(rays, tlas_idx=tidx, ray_flags=flags, cull_mask=mask, anyhit_mode=anyhit, threads=8)
        got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE, tlas_idx=tidx.astype(np.int32), ray_flags=flags,
                               cull_mask=mask, anyhit_mode=anyhit)
        info = (seed, case, flags, mask, anyhit)
        assert np.array_equal(got["prim"], expect["prim"]), info
        for k in ("t", "u", "v"):
            assert same_bits_nan(got[k], expect[k]), (info, k)
        assert np.array_equal(ext[:, 0], expect["geometry"]), info
        assert np.array_equal(ext[:, 1], expect["instance"]), info
        assert np.array_equal(ext[:, 2], expect["custom"]), info
        assert np.array_equal(ext[:, 3], expect["hit_kind"]), info
        got_d, _ = run_product(D, rays, rt.TRAVERSAL_ORDERED_WIDE, tlas_idx=tidx.astype(np.int32), ray_flags=flags,
                               cull_mask=mask, anyhit_mode=anyhit)
        got_h, _ = run_product(P, rays, rt.TRAVERSAL_ORDERED_WIDE, tlas_idx=tidx.astype(np.int32), ray_flags=flags,
                               cull_mask=mask, anyhit_mode=anyhit)
        assert np.array_equal(got_d.view(np.uint8), got_h.view(np.uint8)), (info, "device build")
        first_hit = bool(flags & rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH) or anyhit == 1
        exposed = S.nan_exposure(rays, tlas_idx=tidx, ray_flags=flags, cull_mask=mask, threads=8)
        for traversal in ORDERED_MODES:
            for local in (0, 1):
                got2, _ = run_product(P, rays, traversal, tlas_idx=tidx.astype(np.int32), ray_flags=flags,
                                      cull_mask=mask, anyhit_mode=anyhit, local_stack=local)
                assert np.array_equal(got2["prim"] == orc.MISS, expect["prim"] == orc.MISS), (info, traversal)
                if first_hit:
                    continue
                hit = expect["prim"] != orc.MISS
                same_t = (got2["t"] == expect["t"]) | (np.isnan(got2["t"]) & np.isnan(expect["t"]))
                identical = (got2["prim"] == expect["prim"]) & (~hit | (same_t & (got2["u"] == expect["u"]) &
                                                                        (got2["v"] == expect["v"])))
                identical |= (got2["prim"] == expect["prim"]) & np.isnan(expect["u"]) & np.isnan(got2["u"])
                tie = ~identical & hit & (got2["t"] == expect["t"])
                other = ~identical & ~tie & ~exposed
                assert not other.any(), (info, traversal, local, int(other.sum()), np.nonzero(other)[0][:10])


@pytest.mark.parametrize("seed", range(8))
def test_random_scene_paths(seed, cuda):
    """Multi-bounce diffuse paths (rdn_trace_paths) through the same random scenes: reference
    order equals the oracle's paths bit for bit; the ordered walks diverge only on the few paths
    where a tie or a NaN distance picks another triangle."""
    from test_paths_gpu import product_paths

    sc, rng = random_scene(seed)
    try:
        S = sc.build_oracle()
    except RuntimeError:
        return
    P = sc.build_product()
    rays = random_rays(rng, 8000)
    tidx = rng.integers(0, len(sc.tlas), rays.shape[0]).astype(np.uint32)

    class Batch:
        pass

    b = Batch()
    b.rays, b.tlas_idx = rays, tidx
    exp, seg, _ = orc.trace_paths(S, rays, tidx, max_bounces=4, rr_start=2, seed=seed, threads=8)
    got, gseg, _ = product_paths(P, b, rt.TRAVERSAL_REFERENCE, seed=seed)
    assert gseg == seg, seed
    assert np.array_equal(got["depth_flags"], exp["depth_flags"]), seed
    assert same_bits_nan(got["radiance"], exp["radiance"]), seed
    for traversal in ORDERED_MODES:
        got2, _, _ = product_paths(P, b, traversal, seed=seed)
        same = (got2["depth_flags"] == exp["depth_flags"]) & ((got2["radiance"] == exp["radiance"]) |
                                                              (np.isnan(got2["radiance"]) &
                                                               np.isnan(exp["radiance"])))
        assert same.mean() > 0.99, (seed, traversal, same.mean())


@pytest.mark.parametrize("seed", range(8))
def test_random_scene_wavefront(seed, cuda):
    """The wavefront frame (primary, shadow and bounce rays) over the random scenes, seen by a
    camera outside the scene box: reference order reproduces the oracle's pixel records bit for
    bit; the four-child walk differs only where a tie or a NaN distance picks another triangle."""
    sc, rng = random_scene(seed)
    try:
        S = sc.build_oracle()
    except RuntimeError:
        return
    P = sc.build_product()
    eye = rng.uniform(-1.0, 2.0, 3)
    eye[2] = 3.5
    cam = scenes.PinholeCamera.look_at(tuple(eye), (0.5, 0.5, 0.0), 60.0, 96, 64)
    light = (float(rng.uniform(-1, 2)), float(rng.uniform(-1, 2)), 3.0)
    exp, rays, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), cam.width, cam.height, light, seed, threads=8)
    for traversal in (rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED_WIDE):
        wf = rt.Wavefront(P, cam, light, traversal=traversal)
        wf.run(seed)
        torch.cuda.synchronize()
        got = wf.results()
        assert wf.rays_traced() == tuple(rays)
        same = np.ones(exp.shape[0], bool)
        for f in exp.dtype.names:
            a, b = got[f], exp[f]
            if exp.dtype[f].kind == "f":  # NaN compared as NaN (CPU and GPU NaN payloads differ)
                same &= (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
            else:
                same &= a == b
        if traversal == rt.TRAVERSAL_REFERENCE:
            assert same.all(), (seed, int((~same).sum()))
            continue
        # four-child walk: primaries identical except ties and NaN-exposed rays; with the same
        # primary hit, shadow visibility and direct light are identical; bounce hits may
        # differ at ties or NaN distances, which this check does not track ray by ray
        exposed = S.nan_exposure(scenes.pinhole_rays(cam), threads=8)
        tp = (got["primary_t"] == exp["primary_t"]) | (np.isnan(got["primary_t"]) & np.isnan(exp["primary_t"]))
        same_primary = (got["primary_prim"] == exp["primary_prim"]) & tp
        assert np.all(same_primary | tp | exposed), seed
        ok = same_primary
        assert np.array_equal(got["light"][ok], exp["light"][ok]), seed
        assert same_bits_nan(got["direct"][ok], exp["direct"][ok]), seed
        bt = (got["bounce_t"] == exp["bounce_t"]) | np.isnan(got["bounce_t"]) | np.isnan(exp["bounce_t"])
        bsame = (got["bounce_prim"] == exp["bounce_prim"]) | bt
        assert bsame[ok].mean() > 0.99, (seed, bsame[ok].mean())
