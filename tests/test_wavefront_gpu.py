"""GPU parity of the wavefront executor (rdn_wavefront_shadow_bounce) with the
oracle's restatement of the same pipeline: primary closest hit, shadow ray to a
point light, cosine-weighted bounce from offset origins."""

import numpy as np
import pytest
import torch

from helpers import orc, rt, scenes, single_mesh_scene

pytestmark = pytest.mark.gpu

LIGHT = (0.2, 0.2, 2.0)
# a light just above the field (heights within +-0.092): about 37 % of the
# frame's shadow rays hit the terrain, so first-hit searches end on a hit
LOW_LIGHT = (0.5, 0.5, 0.12)


def run_both(mesh, cam, traversal, sample_index=0, bins=4, refill=0, light=LIGHT, **knobs):
    sc = single_mesh_scene(mesh, bins=bins)
    S, P = sc.build_oracle(), sc.build_product()
    wf = rt.Wavefront(P, cam, light, traversal=traversal, refill=refill)
    for k, v in knobs.items():
        setattr(wf.desc, k, v)
    wf.run(sample_index)
    torch.cuda.synchronize()
    got = wf.results()
    exp, rays, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), cam.width, cam.height, light, sample_index,
                                               threads=4)
    return got, exp, rays, wf.rays_traced()


@pytest.mark.parametrize("sample_index,light", [(0, LIGHT), (5, LIGHT), (2, LOW_LIGHT)])
def test_wavefront_reference_order_bit_identical(sample_index, light, cuda):
    mesh = scenes.heightfield(128, seed=1)
    cam = scenes.heightfield_camera(160, 96)
    got, exp, rays, counts = run_both(mesh, cam, rt.TRAVERSAL_REFERENCE, sample_index, light=light)
    assert counts == tuple(rays)
    assert rays[1] > 0.9 * rays[0]  # the field fills the frame
    for f in exp.dtype.names:
        assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f


@pytest.mark.parametrize("light", [LIGHT, LOW_LIGHT])
@pytest.mark.parametrize("refill", [0, 1, 8, 32])
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE])
def test_wavefront_ordered_matches_except_ties(traversal, refill, light, cuda):
    """refill > 0: the dynamic-fetch secondary schedule."""
    mesh = scenes.heightfield(128, seed=1)
    cam = scenes.heightfield_camera(160, 96)
    got, exp, rays, counts = run_both(mesh, cam, traversal, refill=refill, light=light)
    assert counts == tuple(rays)
    same_primary = (got["primary_prim"] == exp["primary_prim"]) & (got["primary_t"] == exp["primary_t"])
    tie = (~same_primary) & (got["primary_t"] == exp["primary_t"])
    assert np.all(same_primary | tie)
    ok = same_primary
    # with the same primary hit, shadow visibility and the bounce ray are identical;
    # the bounce hit can differ only at an exact tie
    assert np.array_equal(got["light"][ok], exp["light"][ok])
    assert np.array_equal(got["direct"][ok].view(np.uint32), exp["direct"][ok].view(np.uint32))
    bsame = (got["bounce_prim"] == exp["bounce_prim"]) | (got["bounce_t"] == exp["bounce_t"])
    assert np.all(bsame[ok])


@pytest.mark.parametrize("size", [(45, 23), (1, 1), (7, 3)])
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED_WIDE])
def test_ragged_frames(size, traversal, cuda):
    """Frames that are not whole 4x8 tiles: the primary kernel's overhanging
    lanes neither trace nor enqueue, and every record is the oracle's."""
    mesh = scenes.heightfield(64, seed=5)
    cam = scenes.heightfield_camera(*size)
    got, exp, rays, counts = run_both(mesh, cam, traversal, sample_index=1, light=LOW_LIGHT)
    assert counts == tuple(rays)
    assert len(got) == size[0] * size[1]
    if traversal == rt.TRAVERSAL_REFERENCE:
        for f in exp.dtype.names:
            assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f
    else:
        ok = (got["primary_prim"] == exp["primary_prim"]) & (got["primary_t"] == exp["primary_t"])
        assert np.all(ok | (got["primary_t"] == exp["primary_t"]))
        assert np.array_equal(got["light"][ok], exp["light"][ok])


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED_WIDE])
def test_axis_parallel_camera_rays(traversal, cuda):
    """A camera straight above the middle of a 65x65-vertex field: the middle
    column and row of a 33x33 frame have direction components of exactly 0,
    and their origin lies on the grid line x = 0.5, a plane of many node
    boxes. The slab test then meets 0 * inf = NaN, which only the full
    min / max test handles as the reference does; the other rays of the same
    warps test boxes by their near and far planes."""
    mesh = scenes.heightfield(65, seed=4)
    cam = scenes.PinholeCamera.look_at((0.5, 0.5, 2.0), (0.5, 0.5, 0.0), 40.0, 33, 33)
    assert cam.forward[0] == 0.0 and cam.forward[1] == 0.0
    got, exp, rays, counts = run_both(mesh, cam, traversal, sample_index=2, light=LOW_LIGHT)
    assert counts == tuple(rays)
    if traversal == rt.TRAVERSAL_REFERENCE:
        for f in exp.dtype.names:
            assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f
    else:
        same = (got["primary_prim"] == exp["primary_prim"]) & (got["primary_t"] == exp["primary_t"])
        assert np.all(same | (got["primary_t"] == exp["primary_t"]))
        assert np.array_equal(got["primary_flags"], exp["primary_flags"])
        assert np.array_equal(got["light"][same], exp["light"][same])
        bsame = (got["bounce_prim"] == exp["bounce_prim"]) | (got["bounce_t"] == exp["bounce_t"])
        assert np.all(bsame[same])


def test_wavefront_soup_camera(cuda):
    mesh = scenes.triangle_soup(5000, seed=2)
    cam = scenes.soup_camera(64, 48)
    got, exp, rays, counts = run_both(mesh, cam, rt.TRAVERSAL_REFERENCE)
    assert counts == tuple(rays)
    for f in exp.dtype.names:
        assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f


@pytest.mark.parametrize("refill", [1, 8])
def test_wavefront_dynamic_fetch_instanced(refill, cuda):
    """Dynamic fetch through a TLAS of several instances and geometries
    (instance walk, geometry walk and BLAS walk all resumed per lane)."""
    from helpers import instanced_scene

    sc = instanced_scene(seed=0)
    S, P = sc.build_oracle(), sc.build_product()
    cam = scenes.PinholeCamera.look_at((0.5, -1.5, 1.2), (0.5, 0.5, 0.2), 50.0, 96, 64)
    exp, rays, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), 96, 64, LIGHT, 3, tlas=1, threads=4)
    for traversal in (rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE):
        wf = rt.Wavefront(P, cam, LIGHT, traversal=traversal, tlas_uniform=1, refill=refill)
        wf.run(3)
        torch.cuda.synchronize()
        got = wf.results()
        assert wf.rays_traced() == tuple(rays)
        ok = (got["primary_prim"] == exp["primary_prim"]) & (got["primary_t"] == exp["primary_t"])
        assert ok.mean() > 0.99
        assert np.array_equal(got["light"][ok], exp["light"][ok])
        bsame = (got["bounce_prim"] == exp["bounce_prim"]) | (got["bounce_t"] == exp["bounce_t"])
        assert np.all(bsame[ok])


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE])
def test_wavefront_local_memory_stack(traversal, cuda):
    """Traversal stacks in local memory instead of shared memory: same results."""
    mesh = scenes.heightfield(128, seed=1)
    cam = scenes.heightfield_camera(160, 96)
    sc = single_mesh_scene(mesh)
    P = sc.build_product()
    a = rt.Wavefront(P, cam, LIGHT, traversal=traversal)
    a.run(2)
    torch.cuda.synchronize()
    ra = a.results()
    for tier, spec in ((0, 0), (1, 4), (2, 16)):  # register budgets; leaf-postponement thresholds
        b = rt.Wavefront(P, cam, LIGHT, traversal=traversal)
        b.desc.local_stack, b.desc.register_tier, b.desc.speculation = 1, tier, spec
        b.run(2)
        torch.cuda.synchronize()
        rb = b.results()
        assert a.rays_traced() == b.rays_traced()
        same = ra["primary_prim"] == rb["primary_prim"]
        assert same.mean() > 0.999
        assert np.array_equal(ra["primary_t"].view(np.uint32), rb["primary_t"].view(np.uint32))
        assert np.array_equal(ra["light"][same], rb["light"][same])


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED_WIDE])
def test_row_bands_tile_the_frame(traversal, cuda):
    """Bands of a frame (row_offset / frame_height, one per GPU in a split
    frame) give exactly the whole frame's pixel records and ray counts, and the
    oracle's pipeline over the same rows."""
    from rendiation_gb300 import partition

    mesh = scenes.heightfield(128, seed=1)
    cam = scenes.heightfield_camera(160, 96)
    sc = single_mesh_scene(mesh)
    S, P = sc.build_oracle(), sc.build_product()
    whole = rt.Wavefront(P, cam, LIGHT, traversal=traversal)
    whole.run(6)
    torch.cuda.synchronize()
    ref = whole.results()
    parts, counts = [], np.zeros(3, np.int64)
    for r0, r1 in partition.row_bands(cam.height, 3):
        band = rt.Wavefront(P, cam, LIGHT, traversal=traversal, rows=(r0, r1))
        band.run(6)
        torch.cuda.synchronize()
        parts.append(band.results())
        counts += np.array(band.rays_traced())
        exp, _, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), cam.width, cam.height, LIGHT, 6, row0=r0,
                                                row1=r1, threads=4)
        got = parts[-1]
        same = got["primary_prim"] == exp["primary_prim"]
        assert same.mean() > 0.99
        if traversal == rt.TRAVERSAL_REFERENCE:
            for f in exp.dtype.names:
                assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f
    stacked = np.concatenate(parts)
    if traversal == rt.TRAVERSAL_REFERENCE:
        for f in ref.dtype.names:
            assert np.array_equal(stacked[f].view(np.uint32), ref[f].view(np.uint32)), f
    else:  # ordered walks: the same up to exact-distance ties (warps hold other rays)
        same = (stacked["primary_prim"] == ref["primary_prim"]) | (stacked["primary_t"] == ref["primary_t"])
        assert same.all()
    assert tuple(int(x) for x in counts) == whole.rays_traced()


def test_band_outside_the_frame_is_rejected(cuda):
    mesh = scenes.heightfield(16, seed=1)
    P = single_mesh_scene(mesh).build_product()
    cam = scenes.heightfield_camera(32, 16)
    wf = rt.Wavefront(P, cam, LIGHT, rows=(8, 16))
    wf.desc.row_offset = 9  # 9 + 8 rows > 16
    with pytest.raises(Exception):
        wf.run(0)
