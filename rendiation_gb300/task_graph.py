"""Host-side mirror of the reference's device task graph (shader/task-graph).

``DeviceTaskGraphBuildSource`` / ``DeviceTaskGraphExecutor`` keep the
reference's names and meaning (runtime/mod.rs:54-397): ``define_task`` with a
future and ``max_in_flight``, ``capacity``, ``build``,
``dispatch_allocate_init_task``, ``execute(rounds)``,
``read_back_execution_states`` and ``debug_execution``. Futures are EDSL code
in the reference; here they are descriptions of the two programs librdn's
kernels run (include/rdn.h, ``rdn_task_graph_*``):

    BaseShaderFuture().then_spawn_task(task_id).map()      # chain program
    TraceTaskFuture()                                       # ray-trace task

All work runs in CUDA kernels through the C ABI; there is no CPU path.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native
from .raytracing import TRAVERSAL_ORDERED_WIDE, _check

PROGRAM_CHAIN, PROGRAM_TRACE, PROGRAM_EXTERNAL = 0, 1, 2
SPAWN_ZERO, SPAWN_AO_PRIMARY, SPAWN_AO_OCCLUSION = 0, 1, 2
MAP_NONE, MAP_AO_ACCUMULATE, MAP_STORE_CHILD, MAP_STORE_ZERO, MAP_STORE_ONE = 0, 1, 2, 3, 4
INIT_ZERO, INIT_INDEX = 0, 1
ERROR_NO_FREE_SLOT, ERROR_ACTIVE_FULL, ERROR_REMOVED_FULL = 0x1, 0x2, 0x4

# task record states (runtime/task_pool.rs:118-139)
TASK_NOT_EXIST, TASK_NOT_FINISHED_WAKEN, TASK_GO_TO_SLEEP, TASK_NOT_FINISHED_SLEEP, TASK_FINISHED = 0, 1, 2, 3, 4


@dataclass(frozen=True)
class ShaderFuture:
    """A chain BaseShaderFuture -> .then(spawn)* -> .map, or the trace task."""

    program: int = PROGRAM_CHAIN
    spawns: tuple = ()
    map_op: int = MAP_NONE

    def then_spawn_task(self, task_ty: int, payload: int = SPAWN_ZERO) -> "ShaderFuture":
        """.then(|_, then, cx| then.spawner.spawn_new_task(payload, cx.generate_self_as_parent()),
        TaskFuture::new(task_ty)) (future/mod.rs:146-170)."""
        if self.program != PROGRAM_CHAIN:
            raise ValueError("only a chain future can spawn")
        return ShaderFuture(self.program, self.spawns + ((int(task_ty), int(payload)),), self.map_op)

    def map(self, op: int = MAP_NONE) -> "ShaderFuture":
        return ShaderFuture(self.program, self.spawns, int(op))


def BaseShaderFuture() -> ShaderFuture:  # noqa: N802 - the reference's name
    return ShaderFuture()


def TraceTaskFuture() -> ShaderFuture:  # noqa: N802
    return ShaderFuture(program=PROGRAM_TRACE)


def ExternalFuture() -> ShaderFuture:  # noqa: N802
    """A task polled by a CUDA C++ program of the caller's (include/rdn_task.cuh);
    register its launcher with DeviceTaskGraphExecutor.set_poll."""
    return ShaderFuture(program=PROGRAM_EXTERNAL)


@dataclass
class TaskGraphExecutionStates:
    wake_counts: list
    sleep_or_finished_counts: list
    empty_counts: list

    def is_empty(self) -> bool:
        return all(c == 0 for c in self.sleep_or_finished_counts) and all(c == 0 for c in self.wake_counts)


@dataclass
class TaskExecutionDebugInfo:
    active_idx: list
    empty_idx: list
    task_states: list


@dataclass
class _TaskDef:
    future: ShaderFuture
    max_in_flight: int
    payload_words: int


@dataclass
class DeviceTaskGraphBuildSource:
    tasks: list = field(default_factory=list)
    capacity: int = 0

    def define_task(self, future: ShaderFuture, max_in_flight: int, payload_words: int = 1) -> int:
        self.tasks.append(_TaskDef(future, int(max_in_flight), int(payload_words)))
        return len(self.tasks) - 1

    def next_task_idx(self) -> int:
        return len(self.tasks)

    def descs(self):
        arr = (native.TaskGroupDesc * len(self.tasks))()
        for i, t in enumerate(self.tasks):
            d = arr[i]
            d.program = t.future.program
            d.max_in_flight = t.max_in_flight
            d.payload_words = t.payload_words
            d.n_spawn = len(t.future.spawns)
            for k, (ty, op) in enumerate(t.future.spawns):
                d.spawn_type[k] = ty
                d.spawn_op[k] = op
            d.map_op = t.future.map_op
        return arr

    def build(self, system, stream=None) -> "DeviceTaskGraphExecutor":
        return DeviceTaskGraphExecutor(system, self, stream)


class DeviceTaskGraphExecutor:
    def __init__(self, system, source: DeviceTaskGraphBuildSource, stream=None, _handle=None):
        self.system = system
        self._L = system._L
        self.max_in_flight = [t.max_in_flight for t in source.tasks]
        self.capacity = source.capacity
        if _handle is not None:
            self._h = _handle
            return
        h = C.c_void_p()
        descs = source.descs()
        _check(system._h, self._L.rdn_task_graph_create(system._h, descs, len(source.tasks), source.capacity,
                                                        _stream(stream), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.rdn_task_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dispatch_allocate_init_task(self, task_count: int, task_id: int, init: int = INIT_ZERO, stream=None):
        """dispatch_allocate_init_task_by_fn with |_| val(0) (INIT_ZERO) or |id| id (INIT_INDEX)."""
        _check(self.system._h, self._L.rdn_task_graph_dispatch_init(self._h, task_id, task_count, init,
                                                                    _stream(stream)))

    def execute(self, dispatch_round_count: int, env: "native.AoDesc | None" = None, stream=None):
        _check(self.system._h, self._L.rdn_task_graph_execute(self._h, dispatch_round_count,
                                                              C.byref(env) if env is not None else None,
                                                              _stream(stream)))

    def read_back_execution_states(self, stream=None) -> TaskGraphExecutionStates:
        n = len(self.max_in_flight)
        wake, sleep, empty = (np.zeros(n, np.uint32) for _ in range(3))
        _check(self.system._h, self._L.rdn_task_graph_states(self._h, wake.ctypes.data, sleep.ctypes.data,
                                                             empty.ctypes.data, _stream(stream)))
        return TaskGraphExecutionStates([int(x) for x in wake], [int(x) for x in sleep], [int(x) for x in empty])

    def debug_execution(self, stream=None) -> list:
        out = []
        for g, mif in enumerate(self.max_in_flight):
            cap = mif * self.capacity
            active = np.zeros(cap, np.uint32)
            empty = np.zeros(cap, np.uint32)
            states = np.zeros(cap + 1, np.uint32)
            na, ne = C.c_uint32(), C.c_uint32()
            _check(self.system._h, self._L.rdn_task_graph_debug(self._h, g, active.ctypes.data, C.byref(na),
                                                                empty.ctypes.data, C.byref(ne), states.ctypes.data,
                                                                _stream(stream)))
            out.append(TaskExecutionDebugInfo(active[:na.value].tolist(), empty[:ne.value].tolist(), states.tolist()))
        return out

    def capture_until_empty(self, task_count: int, task_id: int, init: int = INIT_ZERO, max_rounds: int = 1024,
                            env: "native.AoDesc | None" = None):
        """dispatch_allocate_init_task then rounds until every group is empty (at
        most max_rounds) as one CUDA graph whose loop the device ends
        (rdn_task_graph_capture). Returns a callable that launches it."""
        g = C.c_void_p()
        _check(self.system._h, self._L.rdn_task_graph_capture(self._h, task_id, task_count, init, max_rounds,
                                                              C.byref(env) if env is not None else None,
                                                              C.byref(g)))
        L = self._L

        class Launch:
            def __call__(self_inner, stream=None):
                st = L.rdn_graph_launch(g, _stream(stream))
                if st != native.RDN_OK:
                    raise native.RdnError(st, "rdn_graph_launch")

            def __del__(self_inner):
                L.rdn_graph_destroy(g)

        return Launch()

    def set_poll(self, task_id: int, fn_ptr: int, user: int | None = None):
        """Registers the launcher (an rdn_task_poll_fn address) of an external program."""
        _check(self.system._h, self._L.rdn_task_graph_set_poll(self._h, task_id, C.c_void_p(fn_ptr),
                                                               C.c_void_p(user) if user else None))

    def check_errors(self, stream=None) -> int:
        f = C.c_uint32()
        _check(self.system._h, self._L.rdn_task_graph_check_errors(self._h, _stream(stream), C.byref(f)))
        return f.value


def _stream(stream):
    import torch

    return C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)


# ---- ambient occlusion (scene/rendering/gpu-ray-tracing/src/feature/ao.rs) ----

def look_at_view_projection_inv(eye, target, up, fov_y_deg, aspect, near=0.01, far=100.0) -> np.ndarray:
    """Inverse of perspective(depth 0..1) * look_at, as 16 floats in the
    reference's Mat4 memory order (columns)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = -view[:3, :3] @ eye
    t = 1.0 / np.tan(np.radians(fov_y_deg) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = t / aspect, t
    proj[2, 2], proj[2, 3] = far / (near - far), near * far / (near - far)
    proj[3, 2] = -1.0
    inv = np.linalg.inv(proj @ view)
    return inv.T.astype(np.float32).reshape(-1)  # column-major


def ao_desc(width, height, view_projection_inv, camera_position, image, sample_count=0, tlas_uniform=0,
            traversal=TRAVERSAL_ORDERED_WIDE, normals=None) -> "native.AoDesc":
    d = native.AoDesc()
    for k in range(16):
        d.view_projection_inv[k] = float(view_projection_inv[k])
    for k in range(3):
        d.camera_position[k] = float(camera_position[k])
    d.width, d.height = width, height
    d.sample_count = sample_count
    d.tlas_uniform = tlas_uniform
    d.traversal = traversal
    d.normals = normals.data_ptr() if normals is not None else None
    d.image = image.data_ptr()
    return d


class AmbientOcclusion:
    """The reference's SceneRayTracingAORenderer on one acceleration-structure
    system: ``render`` adds one sample to ``image`` (RGBA8, width*height*4
    bytes) and advances ``sample_count``. mode "fused" runs the one-kernel
    frame (rdn_ao_render), "graph" the five-group task graph of the reference
    pipeline (rdn_ao_render_graph)."""

    def __init__(self, system, width, height, view_projection_inv, camera_position, traversal=TRAVERSAL_ORDERED_WIDE,
                 tlas_uniform=0, normals=None, mode="fused", block_size=0, speculation=0):
        import torch

        self.system = system
        self.width, self.height = width, height
        self.image = torch.zeros(width * height * 4, dtype=torch.uint8, device="cuda")
        self.vp_inv = np.asarray(view_projection_inv, np.float32)
        self.cam = np.asarray(camera_position, np.float32)
        self.traversal = traversal
        self.tlas_uniform = tlas_uniform
        self.normals = normals
        self.sample_count = 0
        self.mode = mode
        self.block_size = block_size  # fused kernel's threads per block: 32, 64 or 128 (0 = 128)
        self.speculation = speculation  # ordered walks: leaf postponement threshold (0 = wait for the warp)
        self.graph = None
        if mode == "graph":
            h = C.c_void_p()
            _check(system._h, system._L.rdn_ao_pipeline_create(system._h, width, height, _stream(None), C.byref(h)))
            src = DeviceTaskGraphBuildSource(capacity=((width + 3) // 4) * ((height + 7) // 8) * 32)
            for mif in (2, 1, 1, 1, 1):
                src.tasks.append(_TaskDef(ShaderFuture(), mif, 1))
            self.graph = DeviceTaskGraphExecutor(system, src, _handle=h)
        elif mode != "fused":
            raise ValueError("mode is 'fused' or 'graph'")

    def desc(self, counter=None):
        d = ao_desc(self.width, self.height, self.vp_inv, self.cam, self.image, self.sample_count,
                    self.tlas_uniform, self.traversal, self.normals)
        if counter is not None:
            d.sample_counter = counter.data_ptr()
        d.block_size = self.block_size
        d.speculation = self.speculation
        return d

    def capture(self, counter):
        """One frame captured into a CUDA graph (rdn_ao_capture) that reads its
        sample index from `counter` (a CUDA int32 tensor of one element) and
        advances it; returns a callable that replays the frame."""
        d = self.desc(counter)
        g = C.c_void_p()
        pipe = self.graph._h if self.graph is not None else None
        _check(self.system._h, self.system._L.rdn_ao_capture(self.system._h, pipe, C.byref(d), C.byref(g)))
        L = self.system._L

        class Frame:
            def __call__(self_inner, stream=None):
                st = L.rdn_graph_launch(g, _stream(stream))
                if st != native.RDN_OK:
                    raise native.RdnError(st, "rdn_graph_launch")

            def __del__(self_inner):
                L.rdn_graph_destroy(g)

        return Frame()

    def render(self, stream=None):
        d = self.desc()
        if self.mode == "fused":
            _check(self.system._h, self.system._L.rdn_ao_render(self.system._h, C.byref(d), _stream(stream)))
        else:
            _check(self.system._h, self.system._L.rdn_ao_render_graph(self.graph._h, C.byref(d), _stream(stream)))
        self.sample_count += 1

    def reset_sample(self):
        self.sample_count = 0
        self.image.zero_()

    def result(self) -> np.ndarray:
        return self.image.cpu().numpy().reshape(self.height, self.width, 4)
