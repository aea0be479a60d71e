"""GPU parity of the watertight triangle test (RDN_INTERSECT_WATERTIGHT: Woop,
Benthin and Wald 2013, with Ize's conservative box test) against the oracle's
twin of the same test, and its differences from the reference's formula
(geometry/mod.rs:105-155):

- reference traversal order with the watertight test equals the oracle's
  watertight traversal bit for bit (t, u, v, primitive, instance, hit kind),
  also through instances, masks and every ray flag case;
- the ordered walks equal it except exact-distance ties;
- no ray aimed at a shared edge or vertex of a continuous surface is lost;
- against the reference's formula, every difference is a near-equal distance or
  an edge case (oracle.parity: classes tie / nan / edge, other = 0);
- the wavefront executor with the watertight test equals the oracle's
  watertight pipeline, classified per ray."""

import numpy as np
import pytest

from helpers import edge_rays, orc, rt, scenes, single_mesh_scene, tilted_grid
from oracle import parity
from test_trace_gpu import FLAG_CASES, ORDERED_MODES, assert_bit_identical, inst_scene, run_oracle, run_product  # noqa: F401

pytestmark = pytest.mark.gpu

WT = rt.INTERSECT_WATERTIGHT
LIGHT = (0.2, 0.2, 2.0)


@pytest.fixture(scope="module")
def heightfield():
    mesh = scenes.heightfield(256, seed=1)
    sc = single_mesh_scene(mesh)
    return sc.build_oracle(), sc.build_product(), scenes.pinhole_rays(scenes.heightfield_camera(480, 270))


def test_reference_order_bit_identical(heightfield, cuda):
    S, P, rays = heightfield
    expect, _ = run_oracle(S, rays, watertight=True)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE | WT)
    assert_bit_identical(got, ext, expect)


@pytest.mark.parametrize("traversal", ORDERED_MODES)
def test_ordered_matches_except_ties(heightfield, traversal, cuda):
    S, P, rays = heightfield
    expect, _ = run_oracle(S, rays, watertight=True)
    got, ext = run_product(P, rays, traversal | WT)
    _, c = parity.classify_trace(S, rays, got, ext, expect, exact=True, threads=8)
    assert c["other"] == 0 and c["edge"] == 0, c


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE] + ORDERED_MODES)
def test_differences_from_reference_formula_classified(heightfield, traversal, cuda):
    """GPU watertight results against the oracle with the reference's formula:
    the same triangle for > 99% of rays, every other ray a near tie or an edge."""
    S, P, rays = heightfield
    expect, _ = run_oracle(S, rays)
    got, ext = run_product(P, rays, traversal | WT)
    _, c = parity.classify_trace(S, rays, got, ext, expect, exact=False, threads=8)
    assert c["other"] == 0, c
    assert c["identical"] > 0.99 * c["n"], c


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE] + ORDERED_MODES)
def test_no_leak_through_shared_edges(traversal, cuda):
    mesh = tilted_grid(33)
    sc = single_mesh_scene(mesh)
    P = sc.build_product()
    rays = edge_rays(mesh, 40_000, seed=5)
    got, _ = run_product(P, rays, traversal | WT, ext=False)
    assert (got["prim"] == orc.MISS).sum() == 0
    ref, _ = run_product(P, rays, traversal, ext=False)
    assert (ref["prim"] == orc.MISS).sum() > 0  # the reference's formula loses some


@pytest.mark.parametrize("flags,anyhit", FLAG_CASES)
def test_flags_instances_reference_order(inst_scene, flags, anyhit, cuda):  # noqa: F811
    sc, S, P, rays = inst_scene
    rng = np.random.default_rng(flags * 7 + anyhit)
    tidx = rng.integers(0, 2, rays.shape[0]).astype(np.uint32)
    expect, _ = run_oracle(S, rays, tlas_idx=tidx, ray_flags=flags, anyhit_mode=anyhit, watertight=True)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE | WT, tlas_idx=tidx, ray_flags=flags,
                           anyhit_mode=anyhit)
    assert_bit_identical(got, ext, expect)


@pytest.mark.parametrize("light", [LIGHT, (0.5, 0.5, 0.12)])  # the second light is shadowed by the terrain
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED_WIDE])
def test_wavefront_watertight(traversal, light, cuda):
    import torch

    mesh = scenes.heightfield(128, seed=1)
    cam = scenes.heightfield_camera(160, 96)
    sc = single_mesh_scene(mesh)
    S, P = sc.build_oracle(), sc.build_product()
    wf = rt.Wavefront(P, cam, light, traversal=traversal | WT)
    wf.run(4)
    torch.cuda.synchronize()
    got = wf.results()
    exp, rays, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), cam.width, cam.height, light, 4, threads=8,
                                               watertight=True)
    assert wf.rays_traced() == tuple(rays)
    if traversal == rt.TRAVERSAL_REFERENCE:
        for f in exp.dtype.names:
            assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f
    res = parity.classify_wavefront(S, cam, cam.width, cam.height, light, got, exp, 4, watertight=True, threads=8)
    assert res["other"] == 0, res
