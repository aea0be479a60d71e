"""The library through its C ABI alone: tests/c_client.c includes only
include/rdn.h and the CUDA runtime, links librdn.so, and builds, traces and
writes results the way a non-Python host would bind the library. Without a
GPU the client must fail cleanly with an rdn_status; on the GPU its hits
equal the oracle's (reference order bit for bit, the four-child walk except
ties), with the host and the GPU build."""

import os
import struct
import subprocess

import numpy as np
import pytest

from helpers import ROOT, orc, rt, scenes, single_mesh_scene
from rendiation_gb300 import native

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def cuda_lib_dir():
    for d in ("lib64", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib", "lib"):
        p = os.path.join(CUDA, d)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(CUDA, "lib64")


def compile_client(tmp_path) -> str:
    exe = str(tmp_path / "c_client")
    lib_dir = os.path.dirname(native.LIB_PATH)
    cud = cuda_lib_dir()
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Werror", os.path.join(ROOT, "tests", "c_client.c"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           os.path.join(lib_dir, "librdn.so"), "-L", cud, "-lcudart",
           f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{cud}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def write_input(path, mesh, rays):
    idx = mesh.indices if mesh.indices is not None else np.zeros(0, np.uint32)
    with open(path, "wb") as f:
        f.write(struct.pack("<III", mesh.positions.shape[0], idx.size, rays.shape[0]))
        f.write(np.ascontiguousarray(mesh.positions, np.float32).tobytes())
        f.write(np.ascontiguousarray(idx, np.uint32).tobytes())
        f.write(np.ascontiguousarray(rays).view(np.float32).tobytes())


def test_client_compiles_and_fails_cleanly_without_gpu(tmp_path):
    import torch

    exe = compile_client(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the GPU test runs the client")
    mesh = scenes.triangle_soup(50, seed=1)
    write_input(tmp_path / "in.bin", mesh, scenes.pinhole_rays(scenes.soup_camera(8, 8)))
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "1", "0"], capture_output=True,
                       text=True)
    assert r.returncode == 2, (r.returncode, r.stderr)
    assert "rdn_create" in r.stderr and "status" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("traversal,device_build", [(rt.TRAVERSAL_REFERENCE, 0), (rt.TRAVERSAL_REFERENCE, 1),
                                                    (rt.TRAVERSAL_ORDERED_WIDE, 1)])
def test_client_traces_like_the_oracle(tmp_path, traversal, device_build, cuda):
    exe = compile_client(tmp_path)
    mesh = scenes.heightfield(48, seed=6)
    rays = np.concatenate([scenes.pinhole_rays(scenes.heightfield_camera(80, 60)),
                           scenes.sphere_rays(3000, (0, 0, -0.2), (1, 1, 0.5), seed=8)])
    write_input(tmp_path / "in.bin", mesh, rays)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(traversal), str(device_build)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(tmp_path / "out.bin", "rb").read()
    n = rays.shape[0]
    hits = np.frombuffer(raw[:16 * n], np.float32).reshape(n, 4)
    ext = np.frombuffer(raw[16 * n:32 * n], np.uint32).reshape(n, 4)
    flags = struct.unpack("<I", raw[32 * n:32 * n + 4])[0]
    assert flags == 0
    expect, _ = single_mesh_scene(mesh).build_oracle().trace(rays, threads=8)
    prim = hits[:, 3].view(np.uint32)
    if traversal == rt.TRAVERSAL_REFERENCE:
        assert np.array_equal(prim, expect["prim"])
        hit = expect["prim"] != orc.MISS
        for k, name in enumerate(("t", "u", "v")):
            assert np.array_equal(hits[hit, k].view(np.uint32), expect[name][hit].view(np.uint32)), name
        assert np.array_equal(ext[:, 3], expect["hit_kind"])
    else:
        same = (prim == expect["prim"]) | (hits[:, 0] == expect["t"])
        assert same.all()
    assert (expect["prim"] != orc.MISS).mean() > 0.3


@pytest.mark.gpu
@pytest.mark.parametrize("traversal", [rt.TRAVERSAL_REFERENCE, rt.TRAVERSAL_ORDERED_WIDE])
def test_client_renders_a_wavefront_frame_like_the_oracle(tmp_path, traversal, cuda):
    """The encoder-side entry point through the C ABI alone: one frame of the
    path tracer's first bounce (primary, shadow, bounce) with caller-owned
    scratch; reference order equals the oracle's pipeline bit for bit."""
    exe = compile_client(tmp_path)
    mesh = scenes.heightfield(64, seed=2)
    rays = scenes.pinhole_rays(scenes.heightfield_camera(16, 8))
    write_input(tmp_path / "in.bin", mesh, rays)
    cam = scenes.heightfield_camera(96, 64)
    light = (0.2, 0.2, 2.0)
    with open(tmp_path / "frame.bin", "wb") as f:
        f.write(struct.pack("<III", cam.width, cam.height, 9))
        f.write(np.asarray(cam.as_floats(), np.float32).tobytes())
        f.write(np.asarray(light, np.float32).tobytes())
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(traversal), "1",
                        str(tmp_path / "frame.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(tmp_path / "out.bin", "rb").read()
    off = 32 * rays.shape[0] + 4
    npix = cam.width * cam.height
    got = np.frombuffer(raw[off:off + 32 * npix], rt.PIXEL_DTYPE)
    counts = np.frombuffer(raw[off + 32 * npix:off + 32 * npix + 12], np.uint32)
    flags = struct.unpack("<I", raw[off + 32 * npix + 12:off + 32 * npix + 16])[0]
    assert flags == 0
    S = single_mesh_scene(mesh).build_oracle()
    exp, n_rays, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), cam.width, cam.height, light, 9, threads=8)
    assert [int(x) for x in counts] == n_rays
    if traversal == rt.TRAVERSAL_REFERENCE:
        for f in exp.dtype.names:
            assert np.array_equal(got[f].view(np.uint32), exp[f].view(np.uint32)), f
    else:
        from oracle import parity

        assert parity.classify_wavefront(S, cam, cam.width, cam.height, light, got, exp, 9, threads=8)["other"] == 0


@pytest.mark.gpu
def test_client_path_traces_like_the_oracle(tmp_path, cuda):
    """rdn_path_tracing_render through the C ABI alone (the wavefront schedule
    with caller scratch, one directional light, the default material): the
    reference order's RGBA8 image equals the oracle's byte for byte."""
    from rendiation_gb300 import path_tracing as pt
    from rendiation_gb300 import task_graph as tg

    exe = compile_client(tmp_path)
    mesh = scenes.heightfield(64, seed=2)
    rays = scenes.pinhole_rays(scenes.heightfield_camera(16, 8))
    write_input(tmp_path / "in.bin", mesh, rays)
    cam = scenes.heightfield_camera(24, 16)
    light = (0.2, 0.2, 2.0)
    with open(tmp_path / "frame.bin", "wb") as f:
        f.write(struct.pack("<III", cam.width, cam.height, 1))
        f.write(np.asarray(cam.as_floats(), np.float32).tobytes())
        f.write(np.asarray(light, np.float32).tobytes())
    W, H = 40, 28
    eye = (0.5, -0.45, 0.75)
    vp = tg.look_at_view_projection_inv(eye, (0.5, 0.5, 0.0), (0, 0, 1), 45.0, W / H)
    sun = pt.directional_light((3.0, 2.5, 2.0), (0.3, 0.2, -1.0))
    with open(tmp_path / "pt.bin", "wb") as f:
        f.write(struct.pack("<IIII", W, H, 2, 3))
        f.write(np.asarray(vp, np.float32).tobytes())
        f.write(np.asarray(eye, np.float32).tobytes())
        f.write(np.asarray(sun["illuminance"], np.float32).tobytes())
        f.write(np.asarray(sun["direction"], np.float32).tobytes())
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), str(rt.TRAVERSAL_REFERENCE), "1",
                        str(tmp_path / "frame.bin"), str(tmp_path / "pt.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = open(tmp_path / "out.bin", "rb").read()
    off = 32 * rays.shape[0] + 4 + 32 * cam.width * cam.height + 16
    img = np.frombuffer(raw[off:off + 4 * W * H], np.uint32)
    counts = np.frombuffer(raw[off + 4 * W * H:off + 4 * W * H + 8], np.uint32)
    flags = struct.unpack("<I", raw[off + 4 * W * H + 8:off + 4 * W * H + 12])[0]
    assert flags == 0
    S = single_mesh_scene(mesh).build_oracle()
    want = np.zeros(W * H, np.uint32)
    n, _ = orc.pt_render(S, vp, eye, W, H, want, lights=[sun], sample_count=2, threads=8)
    assert np.array_equal(img, want)
    assert tuple(int(c) for c in counts) == n
