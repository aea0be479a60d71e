"""GPU BVH build (rdn_build with device_build = 1) against the oracle and the
host build: every flattened array of the reference layout byte-identical,
the same SAH / median-fallback split counts, and bit-identical trace results
in all three traversal orders (which also covers the two-child and four-child
node layouts and the triangle records the device build writes)."""

import numpy as np
import pytest
import torch

from helpers import Scene, instanced_scene, orc, rt, scenes, single_mesh_scene
from test_trace_gpu import run_product

pytestmark = pytest.mark.gpu


def assert_arrays_equal(P, S=None, Q=None):
    for i, name in enumerate(rt.BUILT_ARRAYS):
        got = P.built_array(name)
        if S is not None:
            assert got == S.buffer(i), name
        if Q is not None:
            assert got == Q.built_array(name), name


def assert_same_traces(P, Q, rays, tlas_idx=None):
    for traversal in (rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE):
        for flags in (0, rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH):
            a, ae = run_product(P, rays, traversal, tlas_idx=tlas_idx, ray_flags=flags)
            b, be = run_product(Q, rays, traversal, tlas_idx=tlas_idx, ray_flags=flags)
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (traversal, flags)
            assert np.array_equal(ae, be), (traversal, flags)


def degenerate_soup(n=4000, seed=3):
    """Clustered centres force the BalanceTree median split (Rust select_nth_unstable)."""
    rng = np.random.default_rng(seed)
    c = np.where(rng.random((n, 1, 3)) < 0.97, 0.5, rng.random((n, 1, 3)))
    c = np.round(c * 8) / 8
    return scenes.Mesh((c + rng.uniform(-0.3, 0.3, (n, 3, 3))).astype(np.float32).reshape(-1, 3), None)


CASES = {
    "soup10k": lambda: single_mesh_scene(scenes.triangle_soup(10_000, seed=0)),
    "heightfield96_bin2": lambda: single_mesh_scene(scenes.heightfield(96, seed=3), bins=2),
    "heightfield64_bin1": lambda: single_mesh_scene(scenes.heightfield(64, seed=4), bins=1),
    "soup3k_bin8": lambda: single_mesh_scene(scenes.triangle_soup(3000, seed=5), bins=8),
    "median_fallback": lambda: single_mesh_scene(degenerate_soup(), bins=2),
    "instanced": lambda: instanced_scene(seed=0),
}


@pytest.mark.parametrize("case", list(CASES))
def test_device_build_equals_oracle(case, cuda):
    sc = CASES[case]()
    S = sc.build_oracle()
    P = sc.build_product(device_build=True)
    st = P.build_stats()
    assert st["device_built"] == 1
    assert_arrays_equal(P, S=S)
    ost = S.build_stats()
    assert st["sah_splits"] == ost["sah_splits"]
    assert st["median_fallbacks"] == ost["median_fallbacks"]
    if case == "median_fallback":
        assert st["median_fallbacks"] > 100


@pytest.mark.parametrize("depth", [1, 3, 6])
def test_device_build_depth_limit(depth, cuda):
    sc = single_mesh_scene(scenes.triangle_soup(5000, seed=6))
    S = sc.build_oracle(blas_max_depth=depth)
    P = sc.build_product(device_build=True, blas_max_depth=depth)
    assert_arrays_equal(P, S=S)
    assert P.build_stats()["max_blas_depth"] == depth


def test_device_build_empty_and_multi_geometry(cuda):
    """A BLAS of three geometries (one without triangles) next to a plain BLAS."""
    a = scenes.triangle_soup(700, seed=7)
    b = scenes.heightfield(20, seed=8)
    empty = np.zeros((0, 3), np.float32)
    blas = [[(b.positions, b.indices, 1)], [(a.positions, None, 1), (empty, None, 1), (b.positions, b.indices, 0)]]
    sc = Scene(blas, [[{"blas": 0}, {"blas": 1}]])
    S = sc.build_oracle()
    P = sc.build_product(device_build=True)
    assert_arrays_equal(P, S=S)


def test_device_build_traces_like_host_build(cuda):
    sc = instanced_scene(seed=1)
    P = sc.build_product(device_build=True)
    Q = sc.build_product()
    rays = scenes.sphere_rays(50_000, (-0.5, -0.5, -0.5), (1.5, 1.5, 1.5), seed=9)
    assert_same_traces(P, Q, rays, tlas_idx=(np.arange(rays.shape[0]) % 2).astype(np.int32))


def test_device_build_large_heightfield(cuda):
    """1024^2 heightfield (2,093,058 triangles), the wavefront workload's scene."""
    m = scenes.heightfield(1024, seed=1)
    sc = single_mesh_scene(m)
    P = sc.build_product(device_build=True)
    Q = sc.build_product()
    assert_arrays_equal(P, Q=Q)
    cam = scenes.heightfield_camera(480, 270)
    assert_same_traces(P, Q, scenes.pinhole_rays(cam))
    sp, sq = P.build_stats(), Q.build_stats()
    print(f"\ndevice build {sp['build_seconds']:.4f} s (GPU span {sp['device_seconds']:.4f} s), "
          f"host build {sq['build_seconds']:.4f} s")


def test_device_build_many_soups(cuda):
    """64 soups of log-uniform size in one build: one tree per geometry, built together."""
    sizes = scenes.log_uniform_ints(64, 1_000, 40_000, seed=3)
    meshes = [scenes.triangle_soup(int(n), seed=100 + k, offset=0.05) for k, n in enumerate(sizes)]
    blas = [[(m.positions, None, 1)] for m in meshes]
    sc = Scene(blas, [[{"blas": k}] for k in range(len(meshes))], blas_bin_size=4)
    P = sc.build_product(device_build=True)
    Q = sc.build_product()
    assert_arrays_equal(P, Q=Q)
    rays = scenes.sphere_rays(20_000, (0, 0, 0), (1, 1, 1), seed=4)
    assert_same_traces(P, Q, rays, tlas_idx=(np.arange(rays.shape[0]) % len(meshes)).astype(np.int32))
