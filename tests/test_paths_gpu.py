"""GPU parity of the batched multi-scene path executor (rdn_trace_paths and its
captured CUDA graph) with the oracle's restatement of the same paths."""

import numpy as np
import pytest
import torch

from helpers import Scene, orc, rt, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batched():
    b = scenes.batched_soups(n_scenes=12, tri_range=(500, 3000), ray_range=(300, 3000), seed=7, offset=0.1)
    sc = Scene([[(m.positions, None, 1)] for m in b.meshes], [[{"blas": s}] for s in range(len(b.meshes))])
    return b, sc.build_oracle(), sc.build_product()


def product_paths(P, b, traversal, graph=False, **kw):
    rays = torch.from_numpy(b.rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    tidx = torch.from_numpy(b.tlas_idx.astype(np.int32)).cuda()
    local = kw.pop("local", False)
    speculation = kw.pop("speculation", None)
    paths = rt.Paths(P, rays, tidx, traversal=traversal, **kw)
    if local:
        paths.configure(local_stack=1)
    if speculation is not None:
        paths.configure(speculation=speculation)
    if graph:
        paths.capture()
        paths.launch_graph()
        torch.cuda.synchronize()
        first = paths.results()
        paths.out.fill_(-1.0)
        paths.launch_graph()
    else:
        paths.run()
        first = None
    torch.cuda.synchronize()
    res, seg = paths.results(), paths.segments()
    paths.close()
    return res, seg, first


def test_paths_reference_order_bit_identical(batched, cuda):
    b, S, P = batched
    exp, seg, _ = orc.trace_paths(S, b.rays, b.tlas_idx, max_bounces=4, rr_start=2, seed=11, threads=4)
    got, gseg, _ = product_paths(P, b, rt.TRAVERSAL_REFERENCE, seed=11)
    assert gseg == seg
    assert seg[0] == b.rays.shape[0] and seg[4] > 0  # paths reach the last bounce
    assert np.array_equal(got["depth_flags"], exp["depth_flags"])
    assert np.array_equal(got["radiance"].view(np.uint32), exp["radiance"].view(np.uint32))


def test_paths_graph_replays_identically(batched, cuda):
    b, S, P = batched
    exp, seg, _ = orc.trace_paths(S, b.rays, b.tlas_idx, max_bounces=4, rr_start=2, seed=3, threads=4)
    got, gseg, first = product_paths(P, b, rt.TRAVERSAL_REFERENCE, graph=True, seed=3)
    assert gseg == seg
    assert np.array_equal(first["depth_flags"], got["depth_flags"])
    assert np.array_equal(got["radiance"].view(np.uint32), exp["radiance"].view(np.uint32))


@pytest.mark.parametrize("refill,local", [(0, 0), (0, 1), (1, 0), (8, 0), (0, 4)])
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE])
def test_paths_ordered_matches_except_ties(batched, traversal, refill, local, cuda):
    """refill > 0: the dynamic-fetch schedule (also replayed from a graph);
    local: traversal stacks in local memory."""
    b, S, P = batched
    exp, seg, _ = orc.trace_paths(S, b.rays, b.tlas_idx, max_bounces=4, rr_start=2, seed=5, threads=4)
    got, gseg, first = product_paths(P, b, traversal, graph=refill == 8, seed=5, refill=refill)
    if local == 1:
        got, gseg, first = product_paths(P, b, traversal, graph=True, seed=5, local=True)
    elif local:  # the leaf-postponement threshold instead
        got, gseg, first = product_paths(P, b, traversal, seed=5, speculation=local)
    if first is not None:
        assert (first["depth_flags"] == got["depth_flags"]).mean() > 0.999
    # a path diverges from the oracle only after an exact-distance tie picks another triangle
    same = (got["depth_flags"] == exp["depth_flags"]) & (got["radiance"] == exp["radiance"])
    assert same.mean() > 0.999, same.mean()


@pytest.mark.parametrize("sort_key", [rt.SORT_SCENE_OCTANT, rt.SORT_SCENE_OCTANT_CELL])
def test_paths_sorted_queues_same_results(batched, sort_key, cuda):
    """Regrouping the queues by key changes only the order rays are traced in."""
    b, S, P = batched
    exp, seg, _ = orc.trace_paths(S, b.rays, b.tlas_idx, max_bounces=4, rr_start=2, seed=11, threads=4)
    got, gseg, _ = product_paths(P, b, rt.TRAVERSAL_REFERENCE, seed=11, sort_key=sort_key)
    assert gseg == seg
    assert np.array_equal(got["depth_flags"], exp["depth_flags"])
    assert np.array_equal(got["radiance"].view(np.uint32), exp["radiance"].view(np.uint32))
    got2, _, first = product_paths(P, b, rt.TRAVERSAL_REFERENCE, graph=True, seed=11, sort_key=sort_key)
    assert np.array_equal(got2["depth_flags"], exp["depth_flags"])
    assert np.array_equal(first["depth_flags"], exp["depth_flags"])


def test_paths_no_roulette_no_bounce(batched, cuda):
    b, S, P = batched
    exp, seg, _ = orc.trace_paths(S, b.rays, b.tlas_idx, max_bounces=0, rr_start=99, seed=1, threads=4)
    got, gseg, _ = product_paths(P, b, rt.TRAVERSAL_REFERENCE, max_bounces=0, rr_start=99, seed=1)
    assert gseg == seg == [b.rays.shape[0]]
    assert np.array_equal(got["depth_flags"], exp["depth_flags"])
