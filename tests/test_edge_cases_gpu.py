"""Edge cases on the GPU: degenerate rays (NaN or zero direction, NaN or huge
origin, empty and inverted ranges, rays parallel to grid planes), empty
launches of every entry point, and a bound TLAS with no instances."""

import ctypes as C

import numpy as np
import pytest
import torch

from helpers import Scene, orc, rt, scenes, single_mesh_scene
from rendiation_gb300 import native
from test_trace_gpu import ORDERED_MODES, assert_bit_identical, run_product

pytestmark = pytest.mark.gpu


def degenerate_rays():
    r = np.zeros(12, scenes.RAY_DTYPE)
    r["org"] = [0.5, 0.5, 1.0]
    r["tmin"], r["tmax"] = 0.0, np.inf
    r["dir"] = [0.0, 0.0, -1.0]
    r["dir"][1] = [np.nan, 0.0, -1.0]
    r["dir"][2] = [0.0, 0.0, 0.0]
    r["org"][3] = [np.nan, 0.5, 1.0]
    r["dir"][4] = [1e30, 0.0, -1.0]
    r["org"][5] = [1e30, 0.5, 1.0]
    r["tmin"][6], r["tmax"][6] = 0.5, 0.5          # zero-length range
    r["tmin"][7], r["tmax"][7] = 2.0, 1.0          # inverted range
    r["org"][8], r["dir"][8] = [0.25, 0.25, 0.2], [1.0, 0.0, 0.0]   # along a grid line, inside the field
    r["org"][9], r["dir"][9] = [-1.0, 0.5, 0.0], [1.0, 0.0, 0.0]    # grazing the field from outside
    r["dir"][10] = [0.0, 0.0, 1.0]                                   # away from the field
    r["org"][11], r["dir"][11] = [0.5, 0.5, 1.0], [1e-30, 1e-30, -1.0]  # denormal-sized components
    return r


@pytest.fixture(scope="module")
def field():
    sc = single_mesh_scene(scenes.heightfield(32, seed=1))
    return sc.build_oracle(), sc.build_product()


def test_degenerate_rays_reference_order(field, cuda):
    S, P = field
    rays = degenerate_rays()
    expect, _ = S.trace(rays)
    got, ext = run_product(P, rays, rt.TRAVERSAL_REFERENCE)
    assert_bit_identical(got, ext, expect)


@pytest.mark.parametrize("traversal", ORDERED_MODES)
@pytest.mark.parametrize("local", [0, 1])
def test_degenerate_rays_ordered(field, traversal, local, cuda):
    S, P = field
    rays = degenerate_rays()
    expect, _ = S.trace(rays)
    got, _ = run_product(P, rays, traversal, local_stack=local)
    assert np.array_equal(got["prim"] != orc.MISS, expect["prim"] != orc.MISS)
    hit = expect["prim"] != orc.MISS
    assert np.array_equal(got["t"][hit], expect["t"][hit])


def test_tlas_without_instances(cuda):
    m = scenes.heightfield(16, seed=2)
    sc = Scene([[(m.positions, m.indices, 1)]], [[]])
    P = sc.build_product()
    rays = scenes.pinhole_rays(scenes.heightfield_camera(8, 8))
    for traversal in (rt.TRAVERSAL_REFERENCE, *ORDERED_MODES):
        got, _ = run_product(P, rays, traversal)
        assert np.all(got["prim"] == orc.MISS)


def test_empty_launches(field, cuda):
    """Every entry point accepts an empty launch and writes nothing."""
    S, P = field
    L = native.lib()
    sentinel = torch.full((4, 8), -3.0, device="cuda")
    # wavefront, 0 x 0
    cam = scenes.heightfield_camera(8, 8)
    wf = rt.Wavefront(P, cam, (0.2, 0.2, 2.0))
    wf.desc.camera.width = 0
    wf.desc.camera.height = 0
    wf.run(0)
    # paths, no rays
    paths = rt.Paths(P, sentinel[:0], None, max_bounces=2)
    paths.run()
    # differentiable calls, no rays
    d = native.AttrLossDesc(sentinel.data_ptr(), 0, 0, sentinel.data_ptr(), None, None, None, None,
                            sentinel.data_ptr(), None, None, 1.0, rt.TRAVERSAL_ORDERED, 0, 0)
    assert L.rdn_attr_loss_forward(P._h, C.byref(d), None) == 0
    assert L.rdn_attr_loss_adjoint(P._h, C.byref(d), None) == 0
    dp = native.AttrPathDesc()
    dp.rays, dp.count, dp.segments, dp.attributes = sentinel.data_ptr(), 0, 2, sentinel.data_ptr()
    dp.grad_vertices, dp.grad_scale = sentinel.data_ptr(), 1.0
    assert L.rdn_attr_paths_forward(P._h, C.byref(dp), None) == 0
    assert L.rdn_attr_paths_adjoint(P._h, C.byref(dp), None) == 0
    dp.from_record = 1
    assert L.rdn_attr_paths_adjoint(P._h, C.byref(dp), None) == 0
    # counted trace, no rays
    hits = torch.zeros((1, 4), device="cuda")
    c = P.trace_counted(sentinel[:0], hits)
    assert c["node_visits"] == 0
    torch.cuda.synchronize()
    assert torch.all(sentinel == -3.0)


def test_error_word_reports_and_recovers(cuda):
    """Failure detection without a GPU fault: kernels record conditions in the
    context's error word and return; rdn_check_errors maps them to a status,
    clears the word, and the context keeps working."""
    mesh = scenes.heightfield(64, seed=1)
    sc = single_mesh_scene(mesh)
    S, P = sc.build_oracle(), sc.build_product()
    cam = scenes.heightfield_camera(96, 64)
    wf = rt.Wavefront(P, cam, (0.2, 0.2, 2.0), traversal=rt.TRAVERSAL_ORDERED, refill=8)
    wf.run(1)
    assert P.check_errors() == (0, 0)
    # a ray naming an unbound TLAS misses and is flagged, status stays OK
    rays = scenes.pinhole_rays(cam)[:64]
    got, _ = run_product(P, rays, rt.TRAVERSAL_ORDERED, tlas_idx=np.full(64, 7, np.int32))
    assert np.all(got["prim"] == orc.MISS)
    st, flags = P.check_errors()
    assert st == 0 and flags == native.ERROR_BAD_TLAS_INDEX
    assert P.check_errors() == (0, 0)  # cleared
    # a tiny iteration cap stops the dynamic-fetch warps: RDN_ERR_TIMEOUT, no hang, no fault
    P.set_iteration_limit(2)
    wf.run(1)
    st, flags = P.check_errors()
    assert st == -6 and flags & native.ERROR_ITERATION_LIMIT  # RDN_ERR_TIMEOUT
    # back to the built-in cap: the same frame completes and matches the oracle
    P.set_iteration_limit(0)
    wf.run(1)
    assert P.check_errors() == (0, 0)
    exp, _, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), 96, 64, (0.2, 0.2, 2.0), 1, threads=4)
    got = wf.results()
    same = got["primary_prim"] == exp["primary_prim"]
    assert same.mean() > 0.999
    assert np.array_equal(got["light"][same], exp["light"][same])
