"""The allocation-free wavefront entry point (rdn_wavefront_shadow_bounce_static).

Callers that cannot allocate device memory (a host that budgets all device
memory up front, or a foreign-language host that only sees the C ABI) use this
entry point, whose queues live in a static array inside librdn. This file is
named to be collected last: it checks, through the C ABI, that two calls in a
row give the same pixel records as the regular entry point with caller-owned
scratch, and that launches too large for the array are rejected.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from helpers import rt, scenes, single_mesh_scene
from rendiation_gb300 import native

pytestmark = pytest.mark.gpu

LIGHT = (0.2, 0.2, 2.0)


def static_desc(cam, out, counts, sample_index, traversal):
    d = native.WavefrontDesc()
    d.camera = rt.camera_struct(cam)
    for k in range(3):
        d.light[k] = LIGHT[k]
    d.sample_index = sample_index
    d.tlas_uniform = 0
    d.traversal = traversal
    d.block_size = 0
    d.out = out.data_ptr()
    d.scratch = None
    d.scratch_bytes = 0
    d.ray_counts = counts.data_ptr()
    d.phases = 0
    return d


@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_REFERENCE])
def test_static_scratch_matches_caller_scratch(traversal, cuda):
    L = native.lib()
    P = single_mesh_scene(scenes.heightfield(128, seed=1)).build_product()
    stream = torch.cuda.current_stream()
    for call, (w, h, sample) in enumerate([(320, 240, 3), (640, 720, 4)]):
        cam = scenes.heightfield_camera(w, h)
        # regular entry point, caller-owned scratch
        wf = rt.Wavefront(P, cam, LIGHT, traversal=traversal)
        wf.run(sample)
        torch.cuda.synchronize()
        expect = wf.results()
        expect_counts = wf.rays_traced()
        # allocation-free entry point, same inputs
        out = torch.full((w * h, 8), -1, dtype=torch.int32, device="cuda")
        counts = torch.zeros(4, dtype=torch.int32, device="cuda")
        d = static_desc(cam, out, counts, sample, traversal)
        st = L.rdn_wavefront_shadow_bounce_static(P._h, C.byref(d), C.c_void_p(stream.cuda_stream))
        assert st == native.RDN_OK, L.rdn_last_error(P._h).decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(rt.PIXEL_DTYPE).reshape(-1)
        for f in expect.dtype.names:
            assert np.array_equal(got[f].view(np.uint32), expect[f].view(np.uint32)), (call, f)
        c = counts.cpu().numpy()
        assert (int(c[0]), int(c[1]), int(c[2])) == expect_counts


def test_static_scratch_rejects_oversize_and_caller_scratch(cuda):
    L = native.lib()
    P = single_mesh_scene(scenes.heightfield(32, seed=2)).build_product()
    cam = scenes.heightfield_camera(1920, 1080)
    out = torch.empty((8, 8), dtype=torch.int32, device="cuda")
    counts = torch.zeros(4, dtype=torch.int32, device="cuda")
    d = static_desc(cam, out, counts, 0, rt.TRAVERSAL_ORDERED)
    st = L.rdn_wavefront_shadow_bounce_static(P._h, C.byref(d), None)
    assert st == -1  # RDN_ERR_INVALID_ARG
    msg = L.rdn_last_error(P._h).decode()
    assert "static array holds 33554432" in msg
    small = scenes.heightfield_camera(16, 16)
    d = static_desc(small, out, counts, 0, rt.TRAVERSAL_ORDERED)
    d.scratch = out.data_ptr()
    d.scratch_bytes = 1 << 20
    assert L.rdn_wavefront_shadow_bounce_static(P._h, C.byref(d), None) == -1


def test_static_split_phases_match_one_call(cuda):
    """phases = 1 (primary kernel, which fills the static queues) and then
    phases = 2 (secondary kernel, which reads them) in separate calls on one
    stream give the same pixel records as one regular two-phase call."""
    L = native.lib()
    P = single_mesh_scene(scenes.heightfield(96, seed=5)).build_product()
    stream = torch.cuda.current_stream()
    w, h, sample = 256, 192, 7
    cam = scenes.heightfield_camera(w, h)
    wf = rt.Wavefront(P, cam, LIGHT, traversal=rt.TRAVERSAL_ORDERED)
    wf.run(sample)
    torch.cuda.synchronize()
    expect = wf.results()
    for _ in range(2):
        out = torch.full((w * h, 8), -1, dtype=torch.int32, device="cuda")
        counts = torch.zeros(4, dtype=torch.int32, device="cuda")
        for phase in (1, 2):
            d = static_desc(cam, out, counts, sample, rt.TRAVERSAL_ORDERED)
            d.phases = phase
            st = L.rdn_wavefront_shadow_bounce_static(P._h, C.byref(d), C.c_void_p(stream.cuda_stream))
            assert st == native.RDN_OK, L.rdn_last_error(P._h).decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(rt.PIXEL_DTYPE).reshape(-1)
        for f in expect.dtype.names:
            assert np.array_equal(got[f].view(np.uint32), expect[f].view(np.uint32)), f


def test_static_never_builds(cuda):
    """A build allocates, so the allocation-free entry point refuses a structure
    changed since its last build (RDN_ERR_NOT_BUILT) instead of building it."""
    L = native.lib()
    P = single_mesh_scene(scenes.heightfield(32, seed=3)).build_product()
    extra = scenes.triangle_soup(100, seed=4)
    P.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(extra.positions)])
    cam = scenes.heightfield_camera(32, 32)
    out = torch.zeros((32 * 32, 8), dtype=torch.int32, device="cuda")
    counts = torch.zeros(4, dtype=torch.int32, device="cuda")
    d = static_desc(cam, out, counts, 0, rt.TRAVERSAL_ORDERED)
    assert L.rdn_wavefront_shadow_bounce_static(P._h, C.byref(d), None) == -7  # RDN_ERR_NOT_BUILT
    assert "rdn_build" in L.rdn_last_error(P._h).decode()
    P.build(blas_bin_size=4)
    assert L.rdn_wavefront_shadow_bounce_static(P._h, C.byref(d), None) == native.RDN_OK
    torch.cuda.synchronize()
