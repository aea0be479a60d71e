"""GPU parity of the batch trace (rdn_trace) against the oracle.

REFERENCE traversal must equal the oracle bit for bit (t, u, v, primitive,
geometry, instance, custom index, hit kind) and reproduce its node-visit and
triangle-test counts exactly. ORDERED traversal must equal it except hits at
exactly the same distance (ties), which are counted; first-hit queries must
agree on hit/miss.
"""

import numpy as np
import pytest
import torch

from helpers import Scene, classify, instanced_scene, orc, rt, scenes, single_mesh_scene

pytestmark = pytest.mark.gpu

ORDERED_MODES = [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE]


def to_dev(rays: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8).copy()).cuda()


def run_product(P, rays, traversal, tlas_idx=None, ext=True, **kw):
    n = rays.shape[0]
    hits = torch.full((max(n, 1), 4), -7.0, dtype=torch.float32, device="cuda")
    hx = torch.full((max(n, 1), 4), -7, dtype=torch.int32, device="cuda") if ext else None
    ti = None if tlas_idx is None else torch.from_numpy(np.asarray(tlas_idx, np.int32)).cuda()
    P.trace(to_dev(rays) if n else torch.zeros((1, 8), device="cuda"), hits, hx, ti, traversal=traversal, count=n,
            **kw)
    torch.cuda.synchronize()
    got = rt.hits_to_numpy(hits)[:n]
    if ext:
        e = hx.cpu().numpy().view(np.uint32)[:n]
        return got, e
    return got, None


def run_oracle(S, rays, tlas_idx=None, **kw):
    return S.trace(rays, tlas_idx=tlas_idx, threads=4, **kw)


def assert_bit_identical(got, ext, expect):
    assert np.array_equal(got["prim"], expect["prim"])
    hit = expect["prim"] != orc.MISS
    for k in ("t", "u", "v"):
        assert np.array_equal(got[k][hit].view(np.uint32), expect[k][hit].view(np.uint32)), k
    assert np.array_equal(got["t"][~hit], expect["t"][~hit])
    if ext is not None:
        assert np.array_equal(ext[:, 0], expect["geometry"])
        assert np.array_equal(ext[:, 1], expect["instance"])
        assert np.array_equal(ext[:, 2], expect["custom"])
        assert np.array_equal(ext[:, 3], expect["hit_kind"])


@pytest.fixture(scope="module")
def soup():
    """The plain closest-hit workload: 10k-triangle soup, 256x256 pinhole rays."""
    mesh = scenes.triangle_soup(10_000, seed=0)
    sc = single_mesh_scene(mesh)
    return sc, sc.build_oracle(), sc.build_product(), scenes.pinhole_rays(scenes.soup_camera())


def test_soup_reference_order_bit_identical(soup, cuda):
    sc, S, P, rays = soup
    expect, tot = run_oracle(S, rays)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE)
    assert_bit_identical(got, ext, expect)
    assert tot["far_assert"] == 0


@pytest.mark.parametrize("traversal", ORDERED_MODES)
def test_soup_ordered_matches_except_ties(soup, traversal, cuda):
    sc, S, P, rays = soup
    expect, _ = run_oracle(S, rays)
    got, ext = run_product(P, rays, traversal)
    c = classify(got, expect)
    assert c["other"] == 0, c
    assert c["hit_mismatch"] == 0, c


def test_counts_equal_reference_counters(soup, cuda):
    sc, S, P, rays = soup
    _, tot = run_oracle(S, rays)
    hits = torch.zeros((rays.shape[0], 4), device="cuda")
    c = P.trace_counted(to_dev(rays), hits, traversal=rt.TRAVERSAL_REFERENCE)
    assert c["node_visits"] == tot["bvh_visit"]
    assert c["tri_tests"] == tot["tri_visit"]
    assert c["tri_hits"] == tot["tri_hit"]
    for trav in ORDERED_MODES:
        c2 = P.trace_counted(to_dev(rays), hits, traversal=trav)
        # the ordered walks prune with the nearest hit found so far: fewer triangle tests
        assert c2["tri_tests"] <= tot["tri_visit"]


@pytest.mark.parametrize("count", [65_531, 31, 1])
@pytest.mark.parametrize("block", [0, 96])
def test_counts_with_a_partial_last_warp(soup, count, block, cuda):
    """Ray counts that leave the last warp partly empty: the counter reduction
    reads every lane of the warp, so lanes past the count must contribute zero."""
    sc, S, P, rays = soup
    sub = np.ascontiguousarray(rays[:count])
    _, tot = run_oracle(S, sub)
    hits = torch.zeros((count, 4), device="cuda")
    c = P.trace_counted(to_dev(sub), hits, traversal=rt.TRAVERSAL_REFERENCE, block_size=block)
    assert (c["node_visits"], c["tri_tests"], c["tri_hits"]) == (tot["bvh_visit"], tot["tri_visit"], tot["tri_hit"])


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE] + ORDERED_MODES)
def test_heightfield_random_rays(traversal, cuda):
    mesh = scenes.heightfield(128, seed=4)
    sc = single_mesh_scene(mesh, bins=2)
    S, P = sc.build_oracle(), sc.build_product()
    rays = scenes.sphere_rays(20_000, (0, 0, -0.3), (1, 1, 0.6), seed=9)
    expect, _ = run_oracle(S, rays)
    got, ext = run_product(P, rays, traversal)
    if traversal == rt.TRAVERSAL_REFERENCE:
        assert_bit_identical(got, ext, expect)
    else:
        c = classify(got, expect)
        assert c["other"] == 0, c


FLAG_CASES = [
    (rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES, 0),
    (rt.RAY_FLAG_CULL_FRONT_FACING_TRIANGLES, 0),
    (rt.RAY_FLAG_SKIP_TRIANGLES, 0),
    (rt.RAY_FLAG_FORCE_NON_OPAQUE, 0),
    (rt.RAY_FLAG_FORCE_NON_OPAQUE, 2),
    (rt.RAY_FLAG_FORCE_NON_OPAQUE, 1),
    (rt.RAY_FLAG_CULL_OPAQUE, 0),
    (rt.RAY_FLAG_CULL_NON_OPAQUE, 0),
    (rt.RAY_FLAG_FORCE_OPAQUE | rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES, 0),
    (rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH, 0),
]


@pytest.fixture(scope="module")
def inst_scene():
    sc = instanced_scene(seed=1)
    rays = scenes.sphere_rays(12_000, (-0.6, -0.6, -0.6), (1.6, 1.6, 1.2), seed=21)
    return sc, sc.build_oracle(), sc.build_product(), rays


@pytest.mark.parametrize("flags,anyhit", FLAG_CASES)
def test_flags_instances_reference_order(inst_scene, flags, anyhit, cuda):
    sc, S, P, rays = inst_scene
    rng = np.random.default_rng(flags * 7 + anyhit)
    tidx = rng.integers(0, 2, rays.shape[0]).astype(np.uint32)
    for mask in (0xFF, 0x02):
        expect, tot = run_oracle(S, rays, tlas_idx=tidx, ray_flags=flags, cull_mask=mask, anyhit_mode=anyhit)
        got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE, tlas_idx=tidx, ray_flags=flags, cull_mask=mask,
                               anyhit_mode=anyhit)
        assert_bit_identical(got, ext, expect)


@pytest.mark.parametrize("traversal", ORDERED_MODES)
@pytest.mark.parametrize("flags,anyhit", FLAG_CASES)
def test_flags_instances_ordered(inst_scene, flags, anyhit, traversal, cuda):
    sc, S, P, rays = inst_scene
    rng = np.random.default_rng(flags * 7 + anyhit)
    tidx = rng.integers(0, 2, rays.shape[0]).astype(np.uint32)
    expect, _ = run_oracle(S, rays, tlas_idx=tidx, ray_flags=flags, anyhit_mode=anyhit)
    got, ext = run_product(P, rays, traversal, tlas_idx=tidx, ray_flags=flags, anyhit_mode=anyhit)
    first_hit = (flags & rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH) or anyhit == 1
    if first_hit:
        # a first-hit query returns *a* hit: only hit/miss is order-independent
        assert np.array_equal(got["prim"] == orc.MISS, expect["prim"] == orc.MISS)
    else:
        c = classify(got, expect)
        assert c["other"] == 0, c


def test_edge_rays(cuda):
    """Axis-parallel directions (infinite reciprocals), origins on boxes and
    vertices, empty ranges, finite far limits and grazing rays."""
    mesh = scenes.heightfield(16, seed=2)
    sc = single_mesh_scene(mesh, bins=2)
    S, P = sc.build_oracle(), sc.build_product()
    g = np.linspace(0, 1, 16, dtype=np.float32)
    org, dirs, tmin, tmax = [], [], [], []
    for x in g[::3]:
        for y in g[::3]:
            for d in ((0, 0, -1), (0, 0, 1), (1, 0, 0), (0, 1, 0), (0.6, 0.8, 0), (0, 0.6, -0.8)):
                org.append((x, y, 0.5))
                dirs.append(d)
                tmin.append(0.0)
                tmax.append(np.inf)
    for k in range(len(org)):
        if k % 5 == 1:
            tmax[k] = 0.3
        if k % 7 == 2:
            tmin[k], tmax[k] = 0.6, 0.2  # empty range
    r = scenes.make_rays(np.array(org, np.float32), np.array(dirs, np.float32))
    r["tmin"] = np.array(tmin, np.float32)
    r["tmax"] = np.array(tmax, np.float32)
    # vertex-exact origins shot straight down onto the grid
    v = mesh.positions[::17]
    r2 = scenes.make_rays(v + np.float32([0, 0, 1]), np.tile(np.float32([0, 0, -1]), (v.shape[0], 1)))
    rays = np.concatenate([r, r2])
    expect, _ = run_oracle(S, rays)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE)
    assert_bit_identical(got, ext, expect)
    for trav in ORDERED_MODES:
        got2, _ = run_product(P, rays, trav)
        c = classify(got2, expect)
        assert c["other"] == 0, c


def test_empty_batch_and_bad_tlas_index(cuda):
    mesh = scenes.triangle_soup(100, seed=1)
    sc = single_mesh_scene(mesh)
    P = sc.build_product()
    got, _ = run_product(P, np.zeros(0, scenes.RAY_DTYPE), rt.TRAVERSAL_ORDERED)
    assert got.shape[0] == 0
    rays = scenes.pinhole_rays(scenes.soup_camera(8, 8))
    got, ext = run_product(P, rays, rt.TRAVERSAL_ORDERED, tlas_idx=np.full(64, 5, np.uint32))
    assert np.all(got["prim"] == orc.MISS)
    assert np.all(ext[:, 0] == orc.MISS)


def test_rebuild_after_delete(cuda):
    """Lazy rebuild on the next trace after create/delete, as get_or_build_gpu_data does."""
    m1 = scenes.triangle_soup(500, seed=3)
    m2 = scenes.triangle_soup(500, seed=4)
    sc = Scene([[(m1.positions, None, 1)], [(m2.positions, None, 1)]], [[{"blas": 0}], [{"blas": 1}]], bind=[0])
    P = sc.build_product()
    rays = scenes.pinhole_rays(scenes.soup_camera(32, 32))
    a, _ = run_product(P, rays, rt.TRAVERSAL_ORDERED)
    P.bind_tlas([1])
    b, _ = run_product(P, rays, rt.TRAVERSAL_ORDERED)
    sc2 = Scene([[(m1.positions, None, 1)], [(m2.positions, None, 1)]], [[{"blas": 0}], [{"blas": 1}]], bind=[1])
    expect, _ = run_oracle(sc2.build_oracle(), rays)
    assert np.array_equal(b["prim"], expect["prim"])
    assert not np.array_equal(a["prim"], b["prim"])


@pytest.mark.parametrize("traversal", ORDERED_MODES)
def test_local_memory_stack_same_hits(soup, traversal, cuda):
    """Traversal stacks in local memory instead of shared memory: the same hits."""
    sc, S, P, rays = soup
    expect, _ = run_oracle(S, rays)
    got, ext = run_product(P, rays, traversal, local_stack=1)
    c = classify(got, expect)
    assert c["other"] == 0 and c["hit_mismatch"] == 0, c


@pytest.mark.parametrize("flags", [0, rt.RAY_FLAG_FORCE_NON_OPAQUE,
                                   rt.RAY_FLAG_FORCE_NON_OPAQUE | rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH])
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE] + ORDERED_MODES)
def test_anyhit_primitive_mask(inst_scene, flags, traversal, cuda):
    """Data-driven any-hit (RDN_ANYHIT_PRIMITIVE_MASK): a non-opaque hit is
    accepted when the triangle's bit is set in a mask over built triangles."""
    sc, S, P, rays = inst_scene
    ntri = len(P.built_array("indices")) // 12
    rng = np.random.default_rng(31 + flags)
    mask = np.packbits(rng.random(ntri + 31) < 0.6, bitorder="little").view(np.uint8)
    mask = np.frombuffer(np.pad(mask, (0, (-len(mask)) % 4)).tobytes(), np.uint32)
    tidx = rng.integers(0, 2, rays.shape[0]).astype(np.uint32)
    expect, _ = S.trace(rays, tlas_idx=tidx, ray_flags=flags, anyhit_mode=rt.ANYHIT_PRIMITIVE_MASK,
                        anyhit_mask=mask, threads=4)
    d_mask = torch.from_numpy(mask.view(np.int32).copy()).cuda()
    got, ext = run_product(P, rays, traversal, tlas_idx=tidx, ray_flags=flags,
                           anyhit_mode=rt.ANYHIT_PRIMITIVE_MASK, anyhit_mask=d_mask)
    if traversal == rt.TRAVERSAL_REFERENCE:
        assert_bit_identical(got, ext, expect)
    elif flags & rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH:
        assert np.array_equal(got["prim"] == orc.MISS, expect["prim"] == orc.MISS)
    else:
        c = classify(got, expect)
        assert c["other"] == 0, c
    # the mask changes results: with every bit clear non-opaque geometry is never hit
    none, _ = S.trace(rays, tlas_idx=tidx, ray_flags=flags, anyhit_mode=rt.ANYHIT_PRIMITIVE_MASK,
                      anyhit_mask=np.zeros_like(mask), threads=4)
    if flags & rt.RAY_FLAG_FORCE_NON_OPAQUE:
        assert np.all(none["prim"] == orc.MISS)
