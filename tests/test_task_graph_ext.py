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
