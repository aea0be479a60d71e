"""CPU tests of the oracle (the C++ restatement of the reference's CPU
ray-query path): hand-computed intersector cases, the restated Rust selection,
agreement with an FP64 brute-force closest hit, and BVH invariants."""

import numpy as np
import pytest

from helpers import orc, scenes, single_mesh_scene

NODE = np.dtype([("aabb_min", np.float32, 3), ("hit_next", np.uint32), ("aabb_max", np.float32, 3),
                 ("miss_next", np.uint32), ("content_range", np.uint32, 2), ("tail", np.uint32, 2)])


def test_triangle_known_answers():
    # unit right triangle in z=0, ray straight down through (0.25, 0.25)
    v0, v1, v2 = [0, 0, 0], [1, 0, 0], [0, 1, 0]
    s, t, u, v = orc.intersect_triangle([0.25, 0.25, 2.0], [0, 0, -1], 0.0, np.inf, v0, v1, v2)
    # normal = +z, b = n.d = -1 -> sign -1; t = 2; u = weight of v1 = 0.25, v = weight of v2 = 0.25
    assert (s, t, u, v) == (-1.0, 2.0, 0.25, 0.25)
    # from below: b = +1 -> sign +1
    s, t, u, v = orc.intersect_triangle([0.5, 0.25, -3.0], [0, 0, 1], 0.0, np.inf, v0, v1, v2)
    assert (s, t, u, v) == (1.0, 3.0, 0.5, 0.25)
    # outside (u + v > 1)
    assert orc.intersect_triangle([0.75, 0.5, 1.0], [0, 0, -1], 0.0, np.inf, v0, v1, v2)[0] == 0.0
    # range: t = 2 rejected when far < 2, accepted when far == 2 (inclusive)
    assert orc.intersect_triangle([0.25, 0.25, 2.0], [0, 0, -1], 0.0, 1.5, v0, v1, v2)[0] == 0.0
    assert orc.intersect_triangle([0.25, 0.25, 2.0], [0, 0, -1], 0.0, 2.0, v0, v1, v2)[0] == -1.0
    assert orc.intersect_triangle([0.25, 0.25, 2.0], [0, 0, -1], 2.5, 9.0, v0, v1, v2)[0] == 0.0
    # culling: cull_back=False culls b >= 0 ... pass iff cull_back != (b < 0)
    assert orc.intersect_triangle([0.25, 0.25, 2.0], [0, 0, -1], 0.0, 9.0, v0, v1, v2, True, True)[0] == 0.0
    assert orc.intersect_triangle([0.25, 0.25, 2.0], [0, 0, -1], 0.0, 9.0, v0, v1, v2, True, False)[0] == -1.0


def test_aabb_known_answers():
    lo, hi = [0, 0, 0], [1, 1, 1]
    assert orc.intersect_aabb([0.5, 0.5, -1], [0, 0, 1], 0.0, np.inf, lo, hi)
    assert not orc.intersect_aabb([0.5, 0.5, -1], [0, 0, -1], 0.0, np.inf, lo, hi)  # behind
    assert not orc.intersect_aabb([0.5, 0.5, -1], [0, 0, 1], 0.0, 0.5, lo, hi)      # t_near 1 >= far
    assert orc.intersect_aabb([0.5, 0.5, 0.5], [1, 0, 0], 0.0, np.inf, lo, hi)      # inside
    # axis-parallel ray exactly in a face plane: (0 - 0) * inf = NaN on that axis, the
    # NaN-ignoring min/max then give t_near = +inf there, so the reference reports a miss
    assert not orc.intersect_aabb([0.0, 0.5, -1], [0, 0, 1], 0.0, np.inf, lo, hi)
    assert orc.intersect_aabb([1e-7, 0.5, -1], [0, 0, 1], 0.0, np.inf, lo, hi)
    # empty box (+inf, -inf) is hit by every ray, as in the reference
    assert orc.intersect_aabb([5, 5, 5], [0.3, 0.4, 0.5], 0.0, np.inf, [np.inf] * 3, [-np.inf] * 3)


@pytest.mark.parametrize("n", [2, 3, 16, 17, 50, 63, 64, 65, 300, 1500, 5000])
def test_select_nth_partitions(n):
    rng = np.random.default_rng(n)
    for keys in (rng.random(n).astype(np.float32), np.round(rng.random(n) * 4).astype(np.float32),
                 np.zeros(n, np.float32), np.arange(n, dtype=np.float32)[::-1].copy()):
        k = n // 2
        idx = orc.select_nth(keys, k)
        assert sorted(idx.tolist()) == list(range(n))
        kk = keys[idx]
        assert np.all(kk[:k] <= kk[k]) and np.all(kk[k + 1:] >= kk[k])


def test_select_small_is_stable_insertion_sort():
    # up to 16 elements the selection sorts by insertion: equal keys keep their order
    keys = np.array([3, 1, 2, 1, 3, 0, 2, 1], np.float32)
    idx = orc.select_nth(keys, 4)
    assert idx.tolist() == [5, 1, 3, 7, 2, 6, 0, 4]


def test_bvh_invariants_and_counters():
    mesh = scenes.triangle_soup(3000, seed=2)
    S = single_mesh_scene(mesh, bins=4).build_oracle()
    nodes = np.frombuffer(S.buffer(orc.BUF_TRI_BVH_FOREST), NODE)
    redirect = np.frombuffer(S.buffer(orc.BUF_INDICES_REDIRECT), np.uint32)
    assert sorted(redirect.tolist()) == list(range(3000))
    tris = mesh.triangles()
    leaf = nodes["hit_next"] == nodes["miss_next"]
    for i in np.nonzero(leaf)[0]:
        a, b = nodes["content_range"][i]
        assert b - a <= 4
        t = tris[redirect[a:b]].reshape(-1, 3)
        if b > a:
            assert np.all(t >= nodes["aabb_min"][i]) and np.all(t <= nodes["aabb_max"][i])
    inner = np.nonzero(~leaf)[0]
    assert np.all(nodes["hit_next"][inner] == inner + 1)  # left child follows its parent in pre-order


def test_oracle_vs_fp64_bruteforce():
    """Closest hits agree with FP64 truth except near-edge / near-tie cases,
    which are counted and bounded."""
    mesh = scenes.triangle_soup(10_000, seed=0)
    S = single_mesh_scene(mesh).build_oracle()
    rays = scenes.pinhole_rays(scenes.soup_camera())
    hits, tot = S.trace(rays, threads=4)
    bf = S.bruteforce_fp64(rays, threads=4)
    hit = hits["prim"] != orc.MISS
    assert np.array_equal(hit, np.isfinite(bf[:, 0]))
    same = hits["prim"][hit] == bf[hit, 3].astype(np.uint32)
    assert same.mean() > 0.999
    rel = np.abs(hits["t"][hit][same] - bf[hit, 0][same]) / np.abs(bf[hit, 0][same])
    assert np.max(rel) < 1e-5
    assert tot["far_assert"] == 0
