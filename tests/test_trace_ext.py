"""Any-hit programs of a caller's own (include/rdn_trace.cuh): tests/trace_ext.cu
traces rays in its own kernels through librdn's traversal with a functor in
place of the built-in any-hit policy. A functor restating
RDN_ANYHIT_ACCEPT_EVEN_PRIMS returns rdn_trace's hits bit for bit in the
reference order and the four-child walk; a procedural alpha test accepts only
hits with u + v < 0.5, and its closest hit equals the nearest such candidate
that a brute-force FP32 pass over every triangle finds."""

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from helpers import ROOT, Scene
from rendiation_gb300 import scenes

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
MODE_THREADED, MODE_WIDE4 = 0, 2


def build_extension(tmp_path) -> str:
    out = str(tmp_path / "libtrace_ext.so")
    cmd = [NVCC, "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC", "-fmad=false",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "rendiation_gb300", "csrc"), os.path.join(ROOT, "tests", "trace_ext.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_trace_header_compiles(tmp_path):
    lib = C.CDLL(build_extension(tmp_path))
    assert lib.trace_custom


def test_trace_params_needs_a_device():
    from rendiation_gb300 import raytracing as rt

    S = rt.AccelerationStructureSystem(device=-1)
    size = C.c_size_t(0)
    assert S._L.rdn_trace_params(S._h, 1, None, C.byref(size)) == 0 and size.value > 0
    buf = (C.c_uint8 * size.value)()
    assert S._L.rdn_trace_params(S._h, 1, buf, C.byref(size)) == -8


@pytest.mark.gpu
@pytest.mark.parametrize("mode,traversal", [(MODE_THREADED, 1), (MODE_WIDE4, 2)])
def test_custom_anyhit(tmp_path, cuda, mode, traversal):
    import torch

    from rendiation_gb300 import raytracing as rt

    lib = C.CDLL(build_extension(tmp_path))
    lib.trace_custom.argtypes = [C.c_void_p] * 3 + [C.c_uint32] * 5 + [C.c_void_p]
    mesh = scenes.heightfield(40, seed=7)
    sc = Scene([[(mesh.positions, mesh.indices, 0)]], [[{"blas": 0}]])  # non-opaque: every hit goes to any-hit
    P = sc.build_product()
    rays = np.concatenate([scenes.pinhole_rays(scenes.heightfield_camera(64, 48)),
                           scenes.sphere_rays(1500, (0, 0, -0.2), (1, 1, 0.5), seed=3)])
    n = rays.shape[0]
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    size = C.c_size_t(0)
    assert P._L.rdn_trace_params(P._h, traversal, None, C.byref(size)) == 0
    prm = (C.c_uint8 * size.value)()
    assert P._L.rdn_trace_params(P._h, traversal, prm, C.byref(size)) == 0
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # restated built-in policy
    out = torch.zeros((n, 4), device="cuda")
    assert lib.trace_custom(prm, d_rays.data_ptr(), out.data_ptr(), n, 0, mode, 0, 0xFF, stream) == 0
    ref = torch.zeros((n, 4), device="cuda")
    P.trace(d_rays, ref, traversal=traversal, anyhit_mode=rt.ANYHIT_ACCEPT_EVEN_PRIMS, local_stack=1)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.cpu().numpy().view(np.uint32))
    # procedural alpha test
    assert lib.trace_custom(prm, d_rays.data_ptr(), out.data_ptr(), n, 1, mode, 0, 0xFF, stream) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    prim = got[:, 3].view(np.uint32)
    hit = prim != 0xFFFFFFFF
    assert hit.mean() > 0.1 and np.all(got[hit, 1] + got[hit, 2] < 0.5)
    # brute force: nearest candidate with u + v < 0.5 over all triangles (f32, the reference's test)
    from oracle import orc

    tris = mesh.positions[mesh.indices.reshape(-1, 3)]
    checked = 0
    for i in np.random.default_rng(5).choice(n, 120, replace=False):
        o, d = rays["org"][i], rays["dir"][i]
        best_t, best_p = np.float32(rays["tmax"][i]), 0xFFFFFFFF
        for k, (a, b, c) in enumerate(tris):
            s_, t_, u_, v_ = orc.intersect_triangle(o, d, float(rays["tmin"][i]), float(best_t), a, b, c)
            if s_ != 0.0 and u_ + v_ < 0.5 and t_ <= best_t:
                best_t, best_p = np.float32(t_), k
        if best_p != 0xFFFFFFFF:
            assert prim[i] == best_p or got[i, 0] == best_t, (i, prim[i], best_p)
            checked += 1
    assert checked > 20
