"""A task program compiled outside librdn (tests/task_graph_ext.cu, built from
include/rdn_task.cuh) running on the device task graph as an
RDN_TASK_PROGRAM_EXTERNAL group: the header compiles for sm_103a on the CPU
side; on the GPU the execution-state counts equal a CPU restatement of the same
program on the task-graph oracle after every round."""

import ctypes as C
import os
import subprocess

import pytest

from helpers import ROOT
from oracle.task_graph_oracle import FINISHED, NO_PARENT, RESOLVED, UNINIT, OracleTaskGraph

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


def build_extension(tmp_path) -> str:
    out = str(tmp_path / "libcountdown.so")
    cmd = [NVCC, "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "rendiation_gb300", "csrc"),
           os.path.join(ROOT, "tests", "task_graph_ext.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_extension_header_compiles(tmp_path):
    lib = C.CDLL(build_extension(tmp_path))
    assert lib.countdown_poll


class CountdownOracle(OracleTaskGraph):
    """The Countdown program of tests/task_graph_ext.cu on the oracle."""

    def __init__(self, capacity, mif):
        super().__init__([((), mif)], capacity)
        self.pl = {}

    def dispatch_index(self, count):
        g = self.groups[0]
        self._prepare(0)
        for i in range(count):
            idx = self._spawn(0, NO_PARENT, NO_PARENT)
            if idx != UNINIT:
                self.pl[idx] = i
        self._commit_alloc(g, g.active)
        self._commit_dealloc(g.empty)

    def _poll_chain(self, gi, idx):
        g = self.groups[0]
        L = g.locals[idx]
        if L[0] == 0:
            L[0] = 1
            n = self.pl[idx]
            if n == 0:
                return True
            h = self._spawn(0, 0, idx)
            if h != UNINIT:
                self.pl[h] = n - 1
            L[1] = h
            return False
        h = L[1]
        if h not in (UNINIT, RESOLVED) and g.state[h] == FINISHED:
            self._cleanup(0, h)
            L[1] = RESOLVED
            return True
        return False


@pytest.mark.gpu
def test_external_program_matches_the_oracle(tmp_path, cuda):
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import task_graph as tg

    lib = C.CDLL(build_extension(tmp_path))
    fn = C.cast(lib.countdown_poll, C.c_void_p).value
    S = rt.AccelerationStructureSystem(device=0)
    src = tg.DeviceTaskGraphBuildSource(capacity=64)
    t = src.define_task(tg.ExternalFuture(), 4)
    exe = src.build(S)
    exe.set_poll(t, fn)
    ora = CountdownOracle(64, 4)
    exe.dispatch_allocate_init_task(12, t, init=tg.INIT_INDEX)
    ora.dispatch_index(12)
    for _ in range(30):
        exe.execute(1)
        ora.execute(1)
        got = exe.read_back_execution_states()
        assert (got.wake_counts, got.sleep_or_finished_counts, got.empty_counts) == ora.read_back_execution_states()
    assert got.is_empty() and exe.check_errors() == 0 and ora.error == 0
    # the same program in a captured graph with the device-ended round loop
    launch = exe.capture_until_empty(12, t, init=tg.INIT_INDEX, max_rounds=100)
    launch()
    assert exe.read_back_execution_states().is_empty()


@pytest.mark.gpu
def test_external_group_needs_its_poll(cuda):
    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import task_graph as tg

    S = rt.AccelerationStructureSystem(device=0)
    src = tg.DeviceTaskGraphBuildSource(capacity=4)
    t = src.define_task(tg.ExternalFuture(), 1)
    exe = src.build(S)
    with pytest.raises(native.RdnError, match="rdn_task_graph_set_poll"):
        exe.execute(1)
    exe.dispatch_allocate_init_task(1, t)


class QueryParams(C.Structure):
    _fields_ = [("rays", C.c_void_p), ("out", C.c_void_p), ("count", C.c_uint32), ("trace_group", C.c_uint32),
                ("closest_group", C.c_uint32), ("miss_group", C.c_uint32), ("ray_flags", C.c_uint32),
                ("cull_mask", C.c_uint32)]


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [0, 0x10])
def test_external_ray_query_pipeline(tmp_path, cuda, flags):
    """External ray generation / closest-hit / miss programs around the built-in
    trace task: in reference order every hit equals the oracle's bit for bit."""
    import numpy as np
    import torch

    from helpers import single_mesh_scene
    from oracle import orc
    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes
    from rendiation_gb300 import task_graph as tg

    lib = C.CDLL(build_extension(tmp_path))
    mesh = scenes.heightfield(40, seed=4)
    rays = np.concatenate([scenes.pinhole_rays(scenes.heightfield_camera(64, 48)),
                           scenes.sphere_rays(2000, (0, 0, -0.2), (1, 1, 0.5), seed=9)])
    n = rays.shape[0]
    sc = single_mesh_scene(mesh)
    S = sc.build_oracle()
    expect, _ = S.trace(rays, ray_flags=flags, cull_mask=0xFF, threads=8)
    P = sc.build_product()
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    src = tg.DeviceTaskGraphBuildSource(capacity=n)
    trace = src.define_task(tg.TraceTaskFuture(), 1, payload_words=16)
    gen = src.define_task(tg.ExternalFuture(), 1, payload_words=1)
    hit = src.define_task(tg.ExternalFuture(), 1, payload_words=24)
    miss = src.define_task(tg.ExternalFuture(), 1, payload_words=16)
    exe = src.build(P)
    prm = QueryParams(d_rays.data_ptr(), out.data_ptr(), n, trace, hit, miss, flags, 0xFF)
    for g, name in ((gen, "raygen_poll"), (hit, "record_hit_poll"), (miss, "record_miss_poll")):
        exe.set_poll(g, C.cast(getattr(lib, name), C.c_void_p).value, C.addressof(prm))
    env = native.AoDesc()
    env.traversal = rt.TRAVERSAL_REFERENCE
    exe.dispatch_allocate_init_task(n, gen, init=tg.INIT_INDEX)
    exe.execute(4, env)
    torch.cuda.synchronize()
    assert exe.read_back_execution_states().is_empty() and exe.check_errors() == 0
    got = out.cpu().numpy()
    prim = got[:, 3].view(np.uint32)
    assert np.array_equal(prim, expect["prim"])
    h = expect["prim"] != orc.MISS
    for k, name in enumerate(("t", "u", "v")):
        assert np.array_equal(got[h, k].view(np.uint32), expect[name][h].view(np.uint32)), name
    assert h.mean() > 0.3
