"""Parity at the benchmark's own sizes, with the launch knobs the benchmark
times (node width, local-memory stacks, register tiers, leaf postponement),
classified per ray by oracle.parity:

- the 1024^2 heightfield (2,093,058 triangles) with the 1920x1080 camera of
  the wavefront benchmark: a band of rows of the primary + shadow + bounce
  frame against the oracle's pipeline on the same rows (the benchmark compares
  the whole frame);
- the 10,000-triangle soup with its 256x256 pinhole camera, every ray.

Every ray must be identical, an exact-distance tie (the reference keeps the
last of equal hits, traverse_cpu.rs:177-184), or NaN-exposed; other = 0."""

import numpy as np
import pytest

from helpers import orc, rt, scenes, single_mesh_scene
from oracle import parity
from test_trace_gpu import run_product

pytestmark = pytest.mark.gpu

LIGHT = (0.2, 0.2, 2.0)
# (primary, secondary) launch knobs: (traversal, block, local_stack, register_tier, speculation)
TIMED_KNOBS = [
    ((rt.TRAVERSAL_ORDERED_WIDE, 64, 1, 1, 16), (rt.TRAVERSAL_ORDERED_WIDE, 128, 1, 1, 4)),
    ((rt.TRAVERSAL_ORDERED_WIDE, 128, 1, 0, 8), (rt.TRAVERSAL_ORDERED, 64, 1, 2, 0)),
    ((rt.TRAVERSAL_ORDERED, 32, 0, 0, 0), (rt.TRAVERSAL_ORDERED_WIDE, 64, 0, 0, 2)),
]
BAND = (470, 590)


@pytest.fixture(scope="module")
def field():
    mesh = scenes.heightfield(1024, seed=1)
    sc = single_mesh_scene(mesh)
    return sc.build_oracle(), sc.build_product(device_build=True)


@pytest.mark.parametrize("knobs", range(len(TIMED_KNOBS)))
def test_heightfield_1080p_band(field, knobs, cuda):
    import torch

    S, P = field
    cam = scenes.heightfield_camera(1920, 1080)
    wf = rt.Wavefront(P, cam, LIGHT)
    wf.configure(*TIMED_KNOBS[knobs])
    wf.run(11)
    torch.cuda.synchronize()
    got = wf.results()[BAND[0] * 1920:BAND[1] * 1920]
    exp, _, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), 1920, 1080, LIGHT, 11, row0=BAND[0], row1=BAND[1],
                                            threads=16)
    res = parity.classify_wavefront(S, cam, 1920, 1080, LIGHT, got, exp, 11, row0=BAND[0], threads=16)
    assert res["other"] == 0, res
    assert res["primary"]["identical"] > 0.999 * res["pixels"], res
    assert res["shadow"]["n"] > 0.9 * res["pixels"] and res["bounce"]["n"] == res["shadow"]["n"], res


@pytest.mark.parametrize("traversal,local", [(rt.TRAVERSAL_ORDERED_WIDE, 1), (rt.TRAVERSAL_ORDERED, 0),
                                             (rt.TRAVERSAL_REFERENCE, 0)])
def test_soup_10k_every_ray(traversal, local, cuda):
    mesh = scenes.triangle_soup(10_000, seed=0)
    sc = single_mesh_scene(mesh)
    S, P = sc.build_oracle(), sc.build_product()
    rays = scenes.pinhole_rays(scenes.soup_camera())
    exp, _ = S.trace(rays, threads=8)
    got, ext = run_product(P, rays, traversal, local_stack=local)
    _, c = parity.classify_trace(S, rays, got, ext, exp, exact=True, threads=8)
    assert c["other"] == 0, c
    if traversal == rt.TRAVERSAL_REFERENCE:
        assert c["identical"] == c["n"], c
    assert (got["prim"] != orc.MISS).sum() == (exp["prim"] != orc.MISS).sum()
