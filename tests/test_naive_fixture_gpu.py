"""The reference's own BVH test scene (naive/test.rs:9-225, restated in tests/naive_fixture.py)
traced by the product on the GPU, with the camera of the reference's CPU test (test.rs:233-296,
range [0, 100]) and of its GPU test (test.rs:298-372, range [0.01, 100]), back faces culled.

Reference-order traversal equals the oracle bit for bit on all five TLAS and reproduces the
committed fixture; the ordered traversals agree except exact-distance ties; the GPU build gives
the host build's arrays. Without culling the sphere's zero-area pole triangles report hits at
distance NaN in the reference's intersector; reference order reproduces those hits too."""

import hashlib

import numpy as np
import pytest

import golden_cases as gc
import naive_fixture as nf
from helpers import classify, orc, rt
from test_trace_gpu import ORDERED_MODES, assert_bit_identical, run_product

pytestmark = pytest.mark.gpu

CULL = rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES
RANGES = {"cpu_test": nf.CPU_TEST_RANGE, "gpu_test": nf.GPU_TEST_RANGE}


@pytest.fixture(scope="module")
def fixture():
    g = gc.load("naive_fixture")
    ms = [gc.scenes.Mesh(np.ascontiguousarray(g[f"{n}_positions"]), np.ascontiguousarray(g[f"{n}_indices"]))
          for n in ("sphere", "torus", "cube")]
    sc = nf.make_scene(ms, transforms=g["transforms"])
    return g, sc, sc.build_oracle(), sc.build_product()


@pytest.mark.parametrize("rng", list(RANGES))
@pytest.mark.parametrize("tlas", range(5))
def test_reference_order_bit_identical(fixture, tlas, rng, cuda):
    g, sc, S, P = fixture
    rays = nf.camera_rays(*RANGES[rng])
    expect, _ = S.trace(rays, tlas_uniform=tlas, ray_flags=CULL, threads=8)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE, tlas_uniform=tlas, ray_flags=CULL)
    assert_bit_identical(got, ext, expect)
    if rng == "cpu_test":
        assert np.array_equal(nf.id_image(got["prim"], orc.MISS), g[f"image{tlas}"])
        sub = got.reshape(nf.H, nf.W)[::4, ::4].reshape(-1)
        ref = g[f"hits{tlas}"]
        assert np.array_equal(sub["prim"], ref["prim"])
        for k in ("t", "u", "v"):
            assert np.array_equal(sub[k].view(np.uint32), ref[k].view(np.uint32)), k


@pytest.mark.parametrize("tlas", range(5))
def test_reference_order_visit_counters(fixture, tlas, cuda):
    """The counters the reference's CPU test prints (test.rs:272-287: BVH visits, triangle
    visits, triangle hits) equal the oracle's."""
    import torch

    g, sc, S, P = fixture
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    _, tot = S.trace(rays, tlas_uniform=tlas, ray_flags=CULL, threads=8)
    d = torch.from_numpy(np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8).copy()).cuda()
    hits = torch.empty((rays.shape[0], 4), device="cuda")
    c = P.trace_counted(d, hits, tlas_uniform=tlas, ray_flags=CULL, traversal=rt.TRAVERSAL_REFERENCE)
    assert (c["node_visits"], c["tri_tests"], c["tri_hits"]) == (tot["bvh_visit"], tot["tri_visit"], tot["tri_hit"])


@pytest.mark.parametrize("traversal", ORDERED_MODES)
@pytest.mark.parametrize("tlas", range(5))
def test_ordered_matches_except_ties(fixture, tlas, traversal, cuda):
    g, sc, S, P = fixture
    rays = nf.camera_rays(*nf.GPU_TEST_RANGE)
    expect, _ = S.trace(rays, tlas_uniform=tlas, ray_flags=CULL, threads=8)
    for local in (0, 1):
        got, _ = run_product(P, rays, traversal, tlas_uniform=tlas, ray_flags=CULL, local_stack=local)
        c = classify(got, expect)
        assert c["other"] == 0 and c["hit_mismatch"] == 0, c


def test_unculled_nan_hits_reference_order(fixture, cuda):
    """Sphere (TLAS 4) without culling: the same primitive on every ray, the same distances and
    barycentrics, NaN where the oracle's is NaN (NaN bit patterns differ between CPUs and GPUs,
    so NaN is compared as NaN)."""
    g, sc, S, P = fixture
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    expect, _ = S.trace(rays, tlas_uniform=4, threads=8)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE, tlas_uniform=4)
    assert np.isnan(expect["t"]).sum() > 0
    assert np.array_equal(got["prim"], expect["prim"])
    for k in ("t", "u", "v"):
        nan = np.isnan(expect[k])
        assert np.array_equal(np.isnan(got[k]), nan), k
        assert np.array_equal(got[k][~nan].view(np.uint32), expect[k][~nan].view(np.uint32)), k
    assert np.array_equal(ext[:, 1], expect["instance"])


@pytest.mark.parametrize("traversal", ORDERED_MODES)
def test_unculled_nan_hits_ordered(fixture, traversal, cuda):
    """Without culling, a NaN distance from a zero-area pole triangle also disables every later
    range test of the ray (comparisons with NaN are false), so which triangle a ray ends with
    depends on the order the walk meets them. The ordered walks may therefore differ from the
    reference on rays that can meet such a triangle (the oracle's nan_exposure); every other ray
    is identical except ties."""
    g, sc, S, P = fixture
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    expect, _ = S.trace(rays, tlas_uniform=4, threads=8)
    got, _ = run_product(P, rays, traversal, tlas_uniform=4)
    nan = S.nan_exposure(rays, tlas_uniform=4)
    assert nan.sum() >= np.isnan(expect["t"]).sum()
    same_t = (got["t"] == expect["t"]) | (np.isnan(got["t"]) & np.isnan(expect["t"]))
    identical = (got["prim"] == expect["prim"]) & same_t
    tie = ~identical & (got["t"] == expect["t"]) & (got["prim"] != orc.MISS)
    assert (~identical & ~nan & ~tie).sum() == 0
    assert np.array_equal(got["prim"] != orc.MISS, expect["prim"] != orc.MISS)
    assert identical.mean() > 0.98


def test_device_build_matches_host_build(fixture, cuda):
    g, sc, S, P = fixture
    D = sc.build_product(device_build=True)
    assert D.build_stats()["device_built"]
    got = [hashlib.sha256(D.built_array(a)).hexdigest() for a in rt.BUILT_ARRAYS]
    assert got == g["digests"].tolist()
    rays = nf.camera_rays(*nf.GPU_TEST_RANGE)
    for tlas in range(5):
        a, _ = run_product(D, rays, rt.TRAVERSAL_ORDERED_WIDE, tlas_uniform=tlas, ray_flags=CULL)
        b, _ = run_product(P, rays, rt.TRAVERSAL_ORDERED_WIDE, tlas_uniform=tlas, ray_flags=CULL)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), tlas


def test_reference_binding(fixture, cuda):
    """TLAS 4 bound alone, as the reference's fixture binds it (test.rs:223-224)."""
    g, sc, S, P = fixture
    alone = nf.make_scene(sc_meshes(sc), transforms=g["transforms"], bind=[nf.TEST_TLAS_IDX])
    A = alone.build_product()
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    got, _ = run_product(A, rays, rt.TRAVERSAL_REFERENCE, ray_flags=CULL)
    assert np.array_equal(nf.id_image(got["prim"], orc.MISS), g[f"image{nf.TEST_TLAS_IDX}"])


def sc_meshes(sc):
    return [gc.scenes.Mesh(b[0][0], b[0][1]) for b in sc.blas]
