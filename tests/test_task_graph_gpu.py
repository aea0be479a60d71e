"""librdn's device task graph against the reference's own task-graph tests
(shader/task-graph/src/test.rs:1-198, through the Python mirror of
DeviceTaskGraphBuildSource / DeviceTaskGraphExecutor) and against the CPU
oracle on seeded random graphs: execution-state counts exact after every
step, per-group state histograms exact, and the pool invariants."""

import random

import numpy as np
import pytest

import helpers  # noqa: F401  (puts the repo root on sys.path)
from oracle.task_graph_oracle import NOT_EXIST, OracleTaskGraph
from rendiation_gb300 import native
from rendiation_gb300 import raytracing as rt
from rendiation_gb300 import task_graph as tg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system(cuda):
    return rt.AccelerationStructureSystem(device=0)


def build(system, groups, capacity):
    src = tg.DeviceTaskGraphBuildSource(capacity=capacity)
    for spawns, mif in groups:
        f = tg.BaseShaderFuture()
        for s in spawns:
            f = f.then_spawn_task(s)
        src.define_task(f.map(), mif)
    return src.build(system)


def test_simple_map(system):
    # test.rs:1-29
    src = tg.DeviceTaskGraphBuildSource()
    test_task = src.define_task(tg.BaseShaderFuture().map(), 2)
    test_task2 = src.define_task(tg.BaseShaderFuture(), 2)
    src.capacity = 12
    exe = src.build(system)
    exe.dispatch_allocate_init_task(3, test_task)
    exe.dispatch_allocate_init_task(4, test_task2)
    info = exe.read_back_execution_states()
    assert info.wake_counts[test_task] == 3 and info.wake_counts[test_task2] == 4
    exe.execute(1)
    info = exe.read_back_execution_states()
    assert info.wake_counts[test_task] == 0 and info.wake_counts[test_task2] == 0
    assert exe.check_errors() == 0


def test_task_graph_then_task_spawn(system):
    # test.rs:31-140, both rounds
    src = tg.DeviceTaskGraphBuildSource(capacity=4)
    test_task = src.define_task(tg.BaseShaderFuture(), 2)
    test_task2 = src.define_task(tg.BaseShaderFuture().then_spawn_task(test_task).map(), 2)
    exe = src.build(system)
    for _ in range(2):
        exe.dispatch_allocate_init_task(3, test_task2)
        info = exe.read_back_execution_states()
        assert info.wake_counts[test_task] == 0 and info.wake_counts[test_task2] == 3
        exe.execute(1)
        info = exe.read_back_execution_states()
        assert info.wake_counts[test_task] == 3
        assert info.sleep_or_finished_counts[test_task] == 0
        assert info.wake_counts[test_task2] == 0
        assert info.sleep_or_finished_counts[test_task2] == 3
        exe.execute(1)
        info = exe.read_back_execution_states()
        assert info.is_empty()
    assert exe.check_errors() == 0


def test_task_graph_then_task_self_spawn_recursive(system):
    # test.rs:142-198
    src = tg.DeviceTaskGraphBuildSource(capacity=4)
    test_task = src.next_task_idx()
    test_task = src.define_task(tg.BaseShaderFuture().then_spawn_task(test_task).map(), 4)
    exe = src.build(system)
    exe.dispatch_allocate_init_task(3, test_task)
    assert exe.read_back_execution_states().wake_counts[test_task] == 3
    for k in (1, 2, 3):
        exe.execute(1)
        info = exe.read_back_execution_states()
        assert info.wake_counts[test_task] == 3
        assert info.sleep_or_finished_counts[test_task] == 3 * k


def test_debug_execution_lists_match_the_oracle(system):
    groups = [((), 2), ((0,), 2)]
    exe = build(system, groups, 4)
    ora = OracleTaskGraph(groups, 4)
    for step in range(3):
        if step == 0:
            exe.dispatch_allocate_init_task(3, 1)
            ora.dispatch_allocate_init_task(3, 1)
        else:
            exe.execute(1)
            ora.execute(1)
        got, want = exe.debug_execution(), ora.debug_execution()
        for g, (a, e, s) in zip(got, want):
            assert sorted(g.active_idx) == sorted(a)
            assert sorted(g.empty_idx) == sorted(e)
            assert g.task_states == s


def histogram(states, cap):
    return np.bincount(np.asarray(states[1:cap + 1]), minlength=5).tolist()


def check_gpu_invariants(infos, caps):
    for info, cap in zip(infos, caps):
        act, emp, st = info.active_idx, info.empty_idx, info.task_states
        assert len(set(act)) == len(act) and len(set(emp)) == len(emp)
        assert not set(act) & set(emp)
        assert all(1 <= i <= cap for i in act + emp)
        assert all(st[i] == tg.TASK_NOT_FINISHED_WAKEN for i in act)
        assert all(st[i] == NOT_EXIST for i in emp)
        live = {i for i in range(1, cap + 1) if st[i] != NOT_EXIST}
        assert live | set(emp) == set(range(1, cap + 1))


@pytest.mark.parametrize("seed", range(16))
def test_random_graphs_match_the_oracle(system, seed):
    rnd = random.Random(1000 + seed)
    n = rnd.randint(1, 6)
    groups = []
    for gi in range(n):
        k = rnd.randint(0, 4) if gi < n - 1 else 0
        groups.append((tuple(rnd.randrange(gi + 1, n) for _ in range(k)), rnd.randint(1, 3)))
    capacity = 32
    caps = [mif * capacity for _, mif in groups]
    exe = build(system, groups, capacity)
    ora = OracleTaskGraph(groups, capacity)
    for _ in range(6):
        g = rnd.randrange(n)
        cnt = rnd.randint(0, 6)
        exe.dispatch_allocate_init_task(cnt, g)
        ora.dispatch_allocate_init_task(cnt, g)
        r = rnd.randint(1, 3)
        exe.execute(r)
        ora.execute(r)
        got = exe.read_back_execution_states()
        wake, sleep, empty = ora.read_back_execution_states()
        assert (got.wake_counts, got.sleep_or_finished_counts, got.empty_counts) == (wake, sleep, empty)
        infos = exe.debug_execution()
        for info, (_, _, st), cap in zip(infos, ora.debug_execution(), caps):
            assert histogram(info.task_states, cap) == histogram(st, cap)
        check_gpu_invariants(infos, caps)
    # nested sequential spawns can need many rounds: run both until the oracle drains
    rounds = 0
    while any(c != 0 for c in ora.read_back_execution_states()[0] + ora.read_back_execution_states()[1]):
        ora.execute(8)
        rounds += 8
        assert rounds < 2000
    exe.execute(rounds)
    assert exe.read_back_execution_states().is_empty()
    assert ora.error == 0 and exe.check_errors() == 0


def test_pool_exhaustion_sets_the_error_flag(system):
    exe = build(system, [((0,), 1)], 4)
    exe.dispatch_allocate_init_task(2, 0)
    exe.execute(5)
    assert exe.check_errors() & tg.ERROR_NO_FREE_SLOT
    info = exe.read_back_execution_states()
    assert info.wake_counts[0] + info.sleep_or_finished_counts[0] + info.empty_counts[0] == 4
    check_gpu_invariants(exe.debug_execution(), [4])


def test_large_fan_out_matches_the_oracle_counts(system):
    # many tiles in the compaction: a two-level chain over 50,000 roots
    groups = [((1, 2), 1), ((2,), 1), ((), 2)]
    exe = build(system, groups, 50_000)
    ora = OracleTaskGraph(groups, 50_000)
    exe.dispatch_allocate_init_task(50_000, 0)
    ora.dispatch_allocate_init_task(50_000, 0)
    for _ in range(6):
        exe.execute(1)
        ora.execute(1)
        got = exe.read_back_execution_states()
        assert (got.wake_counts, got.sleep_or_finished_counts, got.empty_counts) == \
            ora.read_back_execution_states()
    exe.execute(6)
    assert exe.read_back_execution_states().is_empty()


def test_invalid_graphs_are_rejected(system):
    src = tg.DeviceTaskGraphBuildSource(capacity=4)
    src.define_task(tg.BaseShaderFuture().then_spawn_task(5), 1)
    with pytest.raises(native.RdnError, match="does not exist"):
        src.build(system)
    src = tg.DeviceTaskGraphBuildSource(capacity=4)
    src.define_task(tg.TraceTaskFuture(), 1, payload_words=16)
    exe = src.build(system)
    with pytest.raises(native.RdnError, match="environment"):
        exe.execute(1)


@pytest.mark.parametrize("seed", range(6))
def test_captured_drain_loop_empties_the_graph(system, seed):
    """rdn_task_graph_capture: dispatch + a device-ended loop of rounds; one
    launch leaves the graph where the oracle's rounds leave it once no task is
    active: empty, or (where a small pool overflowed) with the same waiting tasks."""
    rnd = random.Random(2000 + seed)
    n = rnd.randint(2, 6)
    groups = []
    for gi in range(n):
        k = rnd.randint(1, 4) if gi < n - 1 else 0
        groups.append((tuple(rnd.randrange(gi + 1, n) for _ in range(k)), rnd.randint(1, 3)))
    exe = build(system, groups, 64)
    ora = OracleTaskGraph(groups, 64)
    cnt = rnd.randint(1, 40)
    ora.dispatch_allocate_init_task(cnt, 0)
    launch = exe.capture_until_empty(cnt, 0, max_rounds=4096)
    launch()
    for _ in range(2000):
        ora.execute(1)
        if not any(ora.read_back_execution_states()[0]):
            break
    got = exe.read_back_execution_states()
    assert (got.wake_counts, got.sleep_or_finished_counts, got.empty_counts) == ora.read_back_execution_states()
    assert bool(exe.check_errors()) == bool(ora.error)
    if not ora.error:
        assert got.is_empty()
        launch()  # a second launch dispatches and drains again
        assert exe.read_back_execution_states().is_empty()


def test_captured_drain_loop_stops_at_max_rounds(system):
    # self-spawning chain (test.rs:142-198): never empties; the loop must stop
    src = tg.DeviceTaskGraphBuildSource(capacity=8)
    t = src.define_task(tg.BaseShaderFuture().then_spawn_task(0).map(), 4)
    exe = src.build(system)
    launch = exe.capture_until_empty(3, t, max_rounds=3)
    launch()
    info = exe.read_back_execution_states()
    assert info.wake_counts[t] == 3 and info.sleep_or_finished_counts[t] == 9
