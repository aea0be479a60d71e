"""The reference's own BVH test scene (naive/test.rs:9-225, restated in tests/naive_fixture.py)
on the CPU: the generators against geometry and the committed fixture, the oracle against
answers computed by hand from the scene's layout and against the fixture, and the product's
host build against the fixture's array digests."""

import hashlib
import math

import numpy as np
import pytest

import golden_cases as gc
import naive_fixture as nf
from helpers import orc, rt

CULL = rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES


@pytest.fixture(scope="module")
def golden():
    return gc.load("naive_fixture")


@pytest.fixture(scope="module")
def oracle():
    return nf.make_scene().build_oracle()


def center_ray_scale():
    """|d| / |d.z| of the ray through pixel (127, 128), the one nearest the optical axis."""
    x = (127 + 0.5) / nf.W * 2 - 1
    y = 1 - (128 + 0.5) / nf.H * 2
    return math.sqrt(x * x + y * y + 1.0)


def test_generators_shape_and_geometry():
    sphere, torus, cube = nf.meshes()
    assert sphere.positions.shape == (33 * 17, 3) and sphere.indices.shape == (32 * 16 * 6,)
    assert torus.positions.shape == (33 * 9, 3) and torus.indices.shape == (32 * 8 * 6,)
    assert cube.positions.shape == (24, 3) and cube.indices.shape == (36,)
    for m in (sphere, torus, cube):
        assert m.indices.max() < m.positions.shape[0]
    r = np.linalg.norm(sphere.positions.astype(np.float64), axis=1)
    assert np.abs(r - 1.0).max() < 1e-6
    t = torus.positions.astype(np.float64)
    ring = np.hypot(t[:, 0], t[:, 1])
    assert np.abs(np.hypot(ring - 1.0, t[:, 2]) - 0.2).max() < 1e-6
    assert np.array_equal(np.abs(cube.positions), np.full((24, 3), 0.5, np.float32))
    # every cube triangle faces outwards (counter-clockwise seen from outside)
    p = cube.positions[cube.indices.reshape(-1, 3)].astype(np.float64)
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    assert (np.einsum("ij,ij->i", n, p.mean(1)) > 0).all()
    assert [len(t) for t in nf.tlas_instances()] == [29, 6, 1, 125, 1]


def test_generators_reproduce_golden(golden):
    for name, m in zip(("sphere", "torus", "cube"), nf.meshes()):
        assert np.array_equal(m.positions.view(np.uint32), golden[f"{name}_positions"].view(np.uint32)), name
        assert np.array_equal(m.indices, golden[f"{name}_indices"]), name
    assert np.array_equal(nf.all_transforms().view(np.uint32), golden["transforms"].view(np.uint32))


def test_oracle_known_answers(oracle):
    """Hits worked out from the layout: the ray nearest the axis meets the front face of the
    cube at (0, 0, -10) at z = -9.5 (TLAS 0) and the nearest cube of the lattice at z = -4.5
    (TLAS 3); it passes through the ring of cubes (TLAS 1) and the torus' hole (TLAS 2); it meets
    the tessellated sphere of radius 5 around (0, 0, -10) just behind z = -5 (TLAS 4)."""
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    c = 128 * nf.W + 127
    s = center_ray_scale()
    hits = [oracle.trace(rays[c:c + 1], tlas_uniform=k, ray_flags=CULL)[0][0] for k in range(5)]
    assert hits[0]["t"] == pytest.approx(9.5 * s, rel=1e-6)
    assert hits[1]["prim"] == orc.MISS and hits[2]["prim"] == orc.MISS
    assert hits[3]["t"] == pytest.approx(4.5 * s, rel=1e-6)
    assert 5.0 * s <= hits[4]["t"] <= 5.0 * s * (1 + 1e-3)
    # TLAS 1: the cube at angle 0 spans y in [3.75, 4.25] at z in [-5.25, -4.75]; the ray through
    # row 20 meets its front face (y = 4.75 * (1 - 20.5 / 128) = 3.99 there)
    row = 20 * nf.W + 127
    h = oracle.trace(rays[row:row + 1], tlas_uniform=1, ray_flags=CULL)[0][0]
    x, y = (127.5 / nf.W) * 2 - 1, 1 - (20.5 / nf.H) * 2
    assert h["t"] == pytest.approx(4.75 * math.sqrt(x * x + y * y + 1), rel=1e-6)


def degenerate_triangles(mesh) -> set[int]:
    p = mesh.positions[mesh.indices.reshape(-1, 3)]
    same = (p[:, 0] == p[:, 1]).all(1) | (p[:, 1] == p[:, 2]).all(1) | (p[:, 0] == p[:, 2]).all(1)
    return set(np.nonzero(same)[0].tolist())


def test_oracle_culling_and_degenerate_pole_triangles(oracle):
    """Rays start outside every closed mesh, so culling back faces keeps the closest distances;
    culling front faces shows the far side of each mesh.

    The UV sphere's first vertex row collapses to its top pole (sin 0 = 0), so 32 of its
    triangles have zero area; at the bottom pole sin(pi) rounds to about -8.7e-8 in FP32 and the
    row keeps that tiny radius. The reference's intersector (geometry/mod.rs:105-155) gives such a triangle a zero
    normal, b = 0 and t = 0 / 0 = NaN, and none of its range or barycentric tests rejects NaN, so
    it reports a hit at distance NaN; the culling test (b < 0 for back-face culling) rejects it.
    Without culling, rays that reach a pole's bounding box therefore return NaN distances, which
    the oracle reproduces."""
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    sphere = nf.meshes()[nf.SPHERE]
    degenerate = degenerate_triangles(sphere)
    assert len(degenerate) == 32
    for k in (0, 4):
        back, _ = oracle.trace(rays, tlas_uniform=k, ray_flags=CULL, threads=4)
        plain, _ = oracle.trace(rays, tlas_uniform=k, threads=4)
        front, _ = oracle.trace(rays, tlas_uniform=k, ray_flags=rt.RAY_FLAG_CULL_FRONT_FACING_TRIANGLES, threads=4)
        hit = back["prim"] != orc.MISS
        assert np.array_equal(hit, plain["prim"] != orc.MISS)
        # the intersector is not watertight: a ray can enter through a face and slip out of its
        # box through an edge (2 of 65536 rays on TLAS 0)
        assert (hit != (front["prim"] != orc.MISS)).sum() <= 4
        assert not np.isnan(back["t"]).any()
        nan = np.isnan(plain["t"])
        assert np.array_equal(back["t"][hit & ~nan], plain["t"][hit & ~nan])
        ok = hit & (front["prim"] != orc.MISS) & ~np.isnan(front["t"])
        assert (front["t"][ok] >= back["t"][ok]).all() and (front["t"][ok] > back["t"][ok]).mean() > 0.95
        if k == 0:
            assert not nan.any()
        else:
            assert nan.sum() > 0 and set(plain["prim"][nan].tolist()) <= degenerate


def test_oracle_nan_exposure(oracle):
    """The oracle's NaN-exposure flag covers every ray whose result is NaN; back-face culling
    (which rejects b = 0) leaves no ray exposed on the sphere."""
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    plain, _ = oracle.trace(rays, tlas_uniform=4, threads=4)
    exposed = oracle.nan_exposure(rays, tlas_uniform=4)
    assert exposed[np.isnan(plain["t"])].all()
    assert exposed.sum() < 0.05 * rays.shape[0]
    assert not oracle.nan_exposure(rays, tlas_uniform=4, ray_flags=CULL).any()
    assert not oracle.nan_exposure(rays, tlas_uniform=0).any()  # cubes seen from outside, no in-plane rays


def test_oracle_reproduces_golden(golden, oracle):
    assert gc.digests_of_oracle(oracle) == golden["digests"].tolist()
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    for k in range(5):
        h, _ = oracle.trace(rays, tlas_uniform=k, ray_flags=CULL, threads=4)
        assert np.array_equal(nf.id_image(h["prim"], orc.MISS), golden[f"image{k}"]), k
        sub = h.reshape(nf.H, nf.W)[::4, ::4].reshape(-1)
        assert np.array_equal(sub.view(np.uint8), golden[f"hits{k}"].view(np.uint8)), k


def test_reference_binding_matches_all_bound(oracle):
    """The reference binds TLAS 4 alone (test.rs:223-224); binding it alone traces the same
    image as selecting it among all five."""
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    alone = nf.make_scene(bind=[nf.TEST_TLAS_IDX]).build_oracle()
    a, _ = alone.trace(rays, tlas_uniform=0, ray_flags=CULL, threads=4)
    b, _ = oracle.trace(rays, tlas_uniform=nf.TEST_TLAS_IDX, ray_flags=CULL, threads=4)
    for k in ("prim", "t", "u", "v"):
        assert np.array_equal(a[k], b[k]), k


def test_product_host_build_matches_golden_digests(golden):
    P = nf.make_scene().build_product(device=-1)
    got = [hashlib.sha256(P.built_array(a)).hexdigest() for a in rt.BUILT_ARRAYS]
    assert got == golden["digests"].tolist()
