"""The task-graph oracle against the reference's own known answers
(shader/task-graph/src/test.rs:1-198), its invariants on seeded random
graphs, and the AO oracle on scenes whose answer is known by hand."""

import random

import numpy as np
import pytest

from helpers import Scene, orc
from oracle.task_graph_oracle import (FINISHED, GO_TO_SLEEP, NOT_EXIST, SLEEP, WAKEN, OracleTaskGraph)

# ---- test.rs:1-29 (test_simple_map) ----


def test_simple_map_known_answer():
    g = OracleTaskGraph([((), 2), ((), 2)], capacity=12)
    g.dispatch_allocate_init_task(3, 0)
    g.dispatch_allocate_init_task(4, 1)
    wake, _, _ = g.read_back_execution_states()
    assert wake == [3, 4]
    g.execute(1)
    wake, _, _ = g.read_back_execution_states()
    assert wake == [0, 0]


# ---- test.rs:31-140 (test_task_graph_then_task_spawn), two rounds ----


def test_then_task_spawn_known_answer():
    g = OracleTaskGraph([((), 2), ((0,), 2)], capacity=4)
    for _ in range(2):
        g.dispatch_allocate_init_task(3, 1)
        wake, sleep, _ = g.read_back_execution_states()
        assert (wake[0], wake[1]) == (0, 3)
        g.execute(1)
        wake, sleep, _ = g.read_back_execution_states()
        assert (wake[0], sleep[0], wake[1], sleep[1]) == (3, 0, 0, 3)
        g.execute(1)
        wake, sleep, _ = g.read_back_execution_states()
        assert (wake[0], sleep[0], wake[1], sleep[1]) == (0, 0, 0, 0)


# ---- test.rs:142-198 (test_task_graph_then_task_self_spawn_recursive) ----


def test_self_spawn_recursive_known_answer():
    g = OracleTaskGraph([((0,), 4)], capacity=4)
    g.dispatch_allocate_init_task(3, 0)
    wake, _, _ = g.read_back_execution_states()
    assert wake == [3]
    for k in (1, 2, 3):
        g.execute(1)
        wake, sleep, _ = g.read_back_execution_states()
        assert (wake[0], sleep[0]) == (3, 3 * k)


def test_first_dispatch_takes_the_top_of_the_empty_pool():
    g = OracleTaskGraph([((), 2), ((0,), 2)], capacity=4)
    g.dispatch_allocate_init_task(3, 1)
    info = g.debug_execution()
    assert sorted(info[1][0]) == [6, 7, 8]
    assert info[1][1] == [1, 2, 3, 4, 5]
    assert [info[1][2][i] for i in (6, 7, 8)] == [WAKEN] * 3
    g.execute(1)
    info = g.debug_execution()
    assert sorted(info[0][0]) == [6, 7, 8]  # children took the top of group 0's pool
    assert [info[1][2][i] for i in (6, 7, 8)] == [SLEEP] * 3


def check_invariants(g: OracleTaskGraph):
    for grp, (active, empty, states) in zip(g.groups, g.debug_execution()):
        assert len(set(active)) == len(active)
        assert len(set(empty)) == len(empty)
        assert not set(active) & set(empty)
        assert all(1 <= i <= grp.cap for i in active + empty)
        assert all(states[i] == WAKEN for i in active)
        assert all(states[i] == NOT_EXIST for i in empty)
        live = {i for i in range(1, grp.cap + 1) if states[i] != NOT_EXIST}
        assert live | set(empty) == set(range(1, grp.cap + 1))
        assert all(states[i] in (WAKEN, SLEEP, FINISHED) for i in live)
        assert GO_TO_SLEEP not in states


def random_graph(seed):
    rnd = random.Random(seed)
    n = rnd.randint(1, 5)
    groups = []
    for gi in range(n):
        # spawn only into later groups, or self-recursion limited by capacity
        k = rnd.randint(0, 3)
        spawns = tuple(rnd.randrange(gi, n) for _ in range(k)) if gi < n - 1 else ()
        groups.append((spawns, rnd.randint(1, 3)))
    return groups, rnd


@pytest.mark.parametrize("seed", range(12))
def test_oracle_invariants_on_random_graphs(seed):
    groups, rnd = random_graph(seed)
    g = OracleTaskGraph(groups, capacity=64)
    for _ in range(4):
        g.dispatch_allocate_init_task(rnd.randint(0, 6), rnd.randrange(len(groups)))
        g.execute(rnd.randint(1, 3))
        check_invariants(g)
    g.execute(40)
    wake, sleep, empty = g.read_back_execution_states()
    if g.error == 0:
        # without self-recursion every chain finishes and leaves the graph empty
        if all(gi not in sp for gi, (sp, _) in enumerate(groups)):
            assert wake == [0] * len(groups) and sleep == [0] * len(groups)


def test_pool_exhaustion_is_an_error_not_a_corruption():
    g = OracleTaskGraph([((0,), 1)], capacity=4)  # recursion past 4 live tasks
    g.dispatch_allocate_init_task(2, 0)
    g.execute(5)
    assert g.error & 0x1
    check_invariants(g)


# ---- AO oracle: known answers ----

def quad(z, size, up=True):
    p = np.array([[-size, -size, z], [size, -size, z], [size, size, z], [-size, size, z]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3] if up else [0, 2, 1, 0, 3, 2], np.uint32)
    return p, idx


def look_down_vp_inv(eye_z):
    from rendiation_gb300.task_graph import look_at_view_projection_inv

    return look_at_view_projection_inv((0, 0, eye_z), (0, 0, 0), (0, 1, 0), 40.0, 1.0, 0.01, 100.0)


def ao_oracle(scene, eye_z, w=16, h=16, samples=1, image=None):
    S = scene.build_oracle()
    img = np.zeros(w * h, np.uint32) if image is None else image
    for s in range(samples):
        orc.ao_render(S, look_down_vp_inv(eye_z), (0, 0, eye_z), w, h, img, sample_count=s, threads=2)
    return img


def test_ao_open_floor_is_unoccluded():
    p, i = quad(0.0, 10.0)
    img = ao_oracle(Scene([[(p, i, 1)]], [[{"blas": 0}]]), 2.0, samples=3)
    assert np.all(img == 0xFFFFFFFF)


def test_ao_covered_floor_is_occluded():
    # floor and ceiling in separate BLAS: a BLAS's box is that of one of its
    # geometries in the reference (see the root-box quirk in the build tests)
    p, i = quad(0.0, 10.0)
    c, ci = quad(0.5, 10.0, up=False)
    img = ao_oracle(Scene([[(p, i, 1)], [(c, ci, 1)]], [[{"blas": 0}, {"blas": 1}]]), 0.25, samples=2)
    assert np.all((img & 0xFF) == 0) and np.all((img >> 24) == 255)


def test_ao_running_average_and_freeze():
    p, i = quad(0.0, 10.0)
    c, ci = quad(0.5, 10.0, up=False)
    scene = Scene([[(p, i, 1)], [(c, ci, 1)]], [[{"blas": 0}, {"blas": 1}]])
    S = scene.build_oracle()
    img = np.full(16 * 16, 0xFFFFFFFF, np.uint32)  # one sample of 1.0 so far
    orc.ao_render(S, look_down_vp_inv(0.25), (0, 0, 0.25), 16, 16, img, sample_count=1)
    assert np.all((img & 0xFF) == 128)  # (1*1 + 0) / 2 = 0.5 -> 127.5 -> 128 (ties to even)
    frozen = img.copy()
    orc.ao_render(S, look_down_vp_inv(0.25), (0, 0, 0.25), 16, 16, img, sample_count=256)
    assert np.array_equal(img, frozen)


def test_ao_camera_miss_writes_one():
    p, i = quad(0.0, 0.01)  # tiny floor: almost every camera ray misses
    img = ao_oracle(Scene([[(p, i, 1)]], [[{"blas": 0}]]), 2.0)
    assert np.all(img == 0xFFFFFFFF)


# ---- C ABI host logic (no device needed) ----

def _create(system, descs, capacity=8):
    import ctypes as C

    from rendiation_gb300 import native

    arr = (native.TaskGroupDesc * max(1, len(descs)))()
    for i, d in enumerate(descs):
        for k, v in d.items():
            if k in ("spawn_type", "spawn_op"):
                for j, x in enumerate(v):
                    getattr(arr[i], k)[j] = x
            else:
                setattr(arr[i], k, v)
    h = C.c_void_p()
    st = system._L.rdn_task_graph_create(system._h, arr, len(descs), capacity, None, C.byref(h))
    msg = system._L.rdn_last_error(system._h).decode()
    return st, msg, h


def test_task_graph_descriptors_are_validated_on_the_host():
    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt

    S = rt.AccelerationStructureSystem(device=-1)
    chain = {"program": 0, "max_in_flight": 1, "payload_words": 1}
    cases = [
        ([], "1 to 16"),
        ([dict(chain)] * 17, "1 to 16"),
        ([dict(chain, max_in_flight=0)], "max_in_flight"),
        ([dict(chain, payload_words=33)], "payload_words"),
        ([dict(chain, n_spawn=1, spawn_type=[3])], "does not exist"),
        ([dict(chain, n_spawn=5)], "at most 4"),
        ([dict(chain, map_op=9)], "unknown map"),
        ([{"program": 1, "max_in_flight": 1, "payload_words": 8}], "at least 16"),
        ([dict(chain, n_spawn=1, spawn_type=[0], spawn_op=[1])], "trace task group"),
        ([dict(chain, map_op=2)], "user payload"),
    ]
    for descs, text in cases:
        st, msg, _ = _create(S, descs)
        assert st == -1 and text in msg, (descs, st, msg)
    # a valid graph on a host-only context: unsupported, not invalid
    st, msg, _ = _create(S, [dict(chain), dict(chain, n_spawn=1, spawn_type=[0])])
    assert st == -8 and "host-only" in msg
    st, msg, _ = _create(S, [dict(chain)], capacity=0)
    assert st == -1 and "capacity" in msg
    assert native.STATUS_NAMES[st] == "RDN_ERR_INVALID_ARG"


def test_ao_entry_points_need_a_device():
    import ctypes as C

    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt

    S = rt.AccelerationStructureSystem(device=-1)
    d = native.AoDesc()
    d.width = d.height = 4
    assert S._L.rdn_ao_render(S._h, C.byref(d), None) == -8
    h = C.c_void_p()
    assert S._L.rdn_ao_pipeline_create(S._h, 4, 4, None, C.byref(h)) == -8
    assert S._L.rdn_ao_pipeline_create(S._h, 0, 4, None, C.byref(h)) == -1
    assert S._L.rdn_task_graph_destroy(None) == 0
