"""The oracle's watertight triangle test (Woop, Benthin and Wald 2013, with the
conservative box test of Ize 2013): hand-computed answers, no ray through a
shared edge or vertex of a continuous surface is lost, NaN distances never
hit, and every difference from the reference's formula (geometry/mod.rs:105-155)
is an equal-distance tie or an edge case on a heightfield under a grazing
camera (oracle only; the GPU twin is tests/test_watertight_gpu.py)."""

import numpy as np

import naive_fixture as nf
from helpers import edge_rays, orc, scenes, single_mesh_scene, tilted_grid
from oracle import parity


def one_triangle_scene(v0, v1, v2):
    pos = np.array([v0, v1, v2], np.float32)
    return single_mesh_scene(scenes.Mesh(pos, np.array([0, 1, 2], np.uint32))).build_oracle()


def trace1(S, o, d, tmin=0.0, tmax=np.inf, flags=0, watertight=True):
    r = scenes.make_rays(np.array([o], np.float32), np.array([d], np.float32), tmin, tmax)
    h, _ = S.trace(r, ray_flags=flags, watertight=watertight)
    return h[0]


def test_known_answers():
    S = one_triangle_scene([0, 0, 0], [1, 0, 0], [0, 1, 0])
    # straight down through (0.25, 0.5): t = 2, weights of v1 / v2 = 0.25 / 0.5, back facing
    # (n = +z, n.d < 0: the reference's sign -1, hit kind 0xFF)
    h = trace1(S, [0.25, 0.5, 2.0], [0, 0, -1])
    assert (h["prim"], h["t"], h["u"], h["v"], h["hit_kind"]) == (0, 2.0, 0.25, 0.5, 0xFF)
    # from below: front facing
    h = trace1(S, [0.5, 0.25, -3.0], [0, 0, 1])
    assert (h["prim"], h["t"], h["u"], h["v"], h["hit_kind"]) == (0, 3.0, 0.5, 0.25, 0xFE)
    # outside, and the range: t = 2 rejected by far < 2 and by near > 2, accepted at far == 2
    assert trace1(S, [0.75, 0.5, 1.0], [0, 0, -1])["prim"] == orc.MISS
    assert trace1(S, [0.25, 0.25, 2.0], [0, 0, -1], tmax=1.5)["prim"] == orc.MISS
    assert trace1(S, [0.25, 0.25, 2.0], [0, 0, -1], tmin=2.5, tmax=9.0)["prim"] == orc.MISS
    assert trace1(S, [0.25, 0.25, 2.0], [0, 0, -1], tmax=2.0)["t"] == 2.0
    # culling and hit kinds follow the reference formula's rules (flag.rs: the
    # cull flags against the sign of n.d) for both sides and both cull flags
    for o, d in (([0.25, 0.25, 2.0], [0, 0, -1]), ([0.25, 0.25, -2.0], [0, 0, 1])):
        for flags in (0x10, 0x20):
            a, b = trace1(S, o, d, flags=flags), trace1(S, o, d, flags=flags, watertight=False)
            assert (a["prim"], a["hit_kind"]) == (b["prim"], b["hit_kind"])
    assert trace1(S, [0.25, 0.25, 2.0], [0, 0, -1], flags=0x10)["prim"] != trace1(
        S, [0.25, 0.25, 2.0], [0, 0, -1], flags=0x20)["prim"]
    # exactly through a vertex and through an edge's midpoint: inclusive, a hit (the
    # rays are tilted: a ray with a zero direction component lying exactly in a box's
    # face plane meets the reference box test's 0 * inf = NaN rule, which skips the box)
    assert trace1(S, [0.25, 0.5, 1.0], [-0.25, -0.5, -1.0])["prim"] == 0
    assert trace1(S, [0.75, 0.25, 1.0], [-0.25, -0.25, -1.0])["prim"] == 0


def test_zero_area_triangle_never_hits():
    """The reference's formula gives t = 0/0 = NaN on a degenerate triangle and
    accepts it; the watertight test has det = 0 there and rejects it."""
    S = one_triangle_scene([0, 0, 0], [1, 0, 0], [2, 0, 0])
    ref = trace1(S, [0.5, 0.5, 1.0], [0, -0.5, -1.0], watertight=False)
    assert ref["prim"] == 0 and np.isnan(ref["t"])
    assert trace1(S, [0.5, 0.5, 1.0], [0, -0.5, -1.0])["prim"] == orc.MISS


def test_no_ray_leaks_through_shared_edges_or_vertices():
    mesh = tilted_grid(33)
    S = single_mesh_scene(mesh).build_oracle()
    rays = edge_rays(mesh, 40_000, seed=3)
    w, _ = S.trace(rays, threads=8, watertight=True)
    r, _ = S.trace(rays, threads=8)
    assert (w["prim"] == orc.MISS).sum() == 0
    # the reference's formula loses a share of them (projected barycentrics, non-conservative boxes)
    assert (r["prim"] == orc.MISS).sum() > 0.02 * len(rays)


def test_differences_from_the_reference_formula_are_ties_or_edges():
    """Grazing camera over a heightfield: every ray where the two formulas
    disagree on hit/miss or triangle is a near-equal distance or lies within
    the reference formula's f32 position error of a triangle edge."""
    mesh = scenes.heightfield(256, seed=1)
    S = single_mesh_scene(mesh).build_oracle()
    rays = scenes.pinhole_rays(scenes.heightfield_camera(480, 270))
    ref, _ = S.trace(rays, threads=8)
    wt, _ = S.trace(rays, threads=8, watertight=True)
    ext = np.stack([wt["geometry"], wt["instance"], wt["custom"], wt["hit_kind"]], 1)
    _, c = parity.classify_trace(S, rays, wt, ext, ref, exact=False, threads=8)
    assert c["other"] == 0, c
    assert c["identical"] > 0.99 * c["n"]
    same = (ref["prim"] == wt["prim"]) & (ref["prim"] != orc.MISS)
    rel = np.abs(wt["t"][same].astype(np.float64) - ref["t"][same]) / ref["t"][same]
    assert rel.max() < 1e-4


def test_reference_fixture_watertight():
    """The reference's own test scene without culling: its sphere's zero-area
    pole triangles give NaN hits under the reference's formula; the watertight
    test reports no NaN distance, and differs only by ties and edge cases."""
    S = nf.make_scene().build_oracle()
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    ref, _ = S.trace(rays, tlas_uniform=4, threads=8)
    wt, _ = S.trace(rays, tlas_uniform=4, threads=8, watertight=True)
    assert np.isnan(ref["t"][ref["prim"] != orc.MISS]).sum() > 0
    assert not np.isnan(wt["t"]).any()
    ext = np.stack([wt["geometry"], wt["instance"], wt["custom"], wt["hit_kind"]], 1)
    _, c = parity.classify_trace(S, rays, wt, ext, ref, exact=False, tlas_uniform=4, threads=8)
    assert c["other"] == 0, c
