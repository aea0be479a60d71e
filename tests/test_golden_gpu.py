"""The product on the GPU against the committed golden fixtures
(tests/golden/*.npz): reference-order traversal reproduces every recorded
result bit for bit, the ordered traversals agree except exact-distance ties,
and the wavefront frame reproduces the recorded pixel records."""

import numpy as np
import pytest
import torch

import golden_cases as gc
from helpers import classify, orc, rt
from test_trace_gpu import ORDERED_MODES, assert_bit_identical, run_product

pytestmark = pytest.mark.gpu


def test_soup_golden_reference_order(cuda):
    g = gc.load("soup1k")
    P = gc.soup_scene(g).build_product()
    rays = gc.rays_of(g)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE)
    assert_bit_identical(got, ext, g["closest"])
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE, ray_flags=rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH)
    assert_bit_identical(got, ext, g["first"])
    d = torch.from_numpy(np.ascontiguousarray(g["rays"])).cuda()
    hits = torch.empty((rays.shape[0], 4), device="cuda")
    c = P.trace_counted(d, hits, traversal=rt.TRAVERSAL_REFERENCE)
    assert c["node_visits"] == int(g["counts"][:, 0].sum())
    assert c["tri_tests"] == int(g["counts"][:, 1].sum())


@pytest.mark.parametrize("traversal", ORDERED_MODES)
def test_soup_golden_ordered(traversal, cuda):
    g = gc.load("soup1k")
    P = gc.soup_scene(g).build_product()
    got, _ = run_product(P, gc.rays_of(g), traversal)
    c = classify(got, g["closest"])
    assert c["other"] == 0 and c["hit_mismatch"] == 0, c
    got, _ = run_product(P, gc.rays_of(g), traversal, ray_flags=rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH)
    assert np.array_equal(got["prim"] != orc.MISS, g["first"]["prim"] != orc.MISS)


@pytest.mark.parametrize("case", range(len(gc.FLAG_CASES)))
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE] + ORDERED_MODES)
def test_instanced_golden(case, traversal, cuda):
    g = gc.load("instanced")
    P = gc.instanced(g).build_product()
    flags, mask = gc.FLAG_CASES[case]
    exp = g[f"hits{case}"]
    got, ext = run_product(P, gc.rays_of(g), traversal, tlas_idx=g["tlas_idx"].astype(np.int32), ray_flags=flags,
                           cull_mask=mask)
    if traversal == rt.TRAVERSAL_REFERENCE:
        assert_bit_identical(got, ext, exp)
    elif flags & rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH:
        assert np.array_equal(got["prim"] != orc.MISS, exp["prim"] != orc.MISS)
    else:
        c = classify(got, exp)
        assert c["other"] == 0 and c["hit_mismatch"] == 0, c


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE] + ORDERED_MODES)
def test_wavefront_golden(traversal, cuda):
    g = gc.load("wavefront")
    P = gc.wavefront_scene(g).build_product()
    cam = gc.camera_of(g, 48, 32)
    wf = rt.Wavefront(P, cam, g["light"], traversal=traversal)
    wf.run(int(g["sample_index"]))
    torch.cuda.synchronize()
    got = wf.results()
    exp = g["pixels"]
    assert list(wf.rays_traced()) == g["ray_counts"].tolist()
    if traversal == rt.TRAVERSAL_REFERENCE:
        for f in exp.dtype.names:
            assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f
    else:
        # a tie can change which triangle a primary hits and so its bounce;
        # the primary distance and the shadow result do not depend on ties
        assert np.array_equal(got["primary_t"].view(np.uint32), exp["primary_t"].view(np.uint32))
        same = got["primary_prim"] == exp["primary_prim"]
        assert same.mean() > 0.99
        for f in exp.dtype.names:
            assert np.array_equal(got[f][same].view(np.uint32), exp[f][same].view(np.uint32)), f
