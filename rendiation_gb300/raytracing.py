"""Host-side mirror of the reference's acceleration-structure and trace interfaces.

``AccelerationStructureSystem`` mirrors ``GPUAccelerationStructureSystemProvider``
(shader/ray-tracing/src/api/backend.rs:120-142) as implemented by the naive SAH
system (shader/ray-tracing/src/backend/wavefront_compute/geometry/naive/mod.rs:560-609):
same method names, same argument meaning, dense handles, deleted slots stay
empty. Queries run through librdn's CUDA kernels via the C ABI (include/rdn.h);
device buffers are torch CUDA tensors (plumbing only).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native

# flags (shader/ray-tracing/src/api/ty.rs:102-159)
RAY_FLAG_NONE = 0x00
RAY_FLAG_FORCE_OPAQUE = 0x01
RAY_FLAG_FORCE_NON_OPAQUE = 0x02
RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH = 0x04
RAY_FLAG_SKIP_CLOSEST_HIT_SHADER = 0x08
RAY_FLAG_CULL_BACK_FACING_TRIANGLES = 0x10
RAY_FLAG_CULL_FRONT_FACING_TRIANGLES = 0x20
RAY_FLAG_CULL_OPAQUE = 0x40
RAY_FLAG_CULL_NON_OPAQUE = 0x80
RAY_FLAG_SKIP_TRIANGLES = 0x100
GEOMETRY_INSTANCE_TRIANGLE_FACING_CULL_DISABLE = 0x1
GEOMETRY_INSTANCE_TRIANGLE_FLIP_FACING = 0x2
GEOMETRY_INSTANCE_FORCE_OPAQUE = 0x4
GEOMETRY_INSTANCE_FORCE_NO_OPAQUE = 0x8
GEOMETRY_FLAG_OPAQUE = 0x1
HIT_KIND_FRONT_FACING_TRIANGLE = 0xFE
HIT_KIND_BACK_FACING_TRIANGLE = 0xFF
MISS = 0xFFFFFFFF

TRAVERSAL_ORDERED = 0
TRAVERSAL_REFERENCE = 1
TRAVERSAL_ORDERED_WIDE = 2
# OR-ed into a traversal value: the watertight triangle test (Woop, Benthin and
# Wald 2013) instead of the reference's formula (geometry/mod.rs:105-155)
INTERSECT_WATERTIGHT = 0x100
SORT_NONE = 0
SORT_SCENE_OCTANT = 1
SORT_SCENE_OCTANT_CELL = 2
ANYHIT_ACCEPT = 0
ANYHIT_ACCEPT_AND_END = 1
ANYHIT_ACCEPT_EVEN_PRIMS = 2
ANYHIT_PRIMITIVE_MASK = 3

# built-array ids of rdn_get_built_array
BUILT_ARRAYS = ["tlas_binding", "tlas_bvh_root", "tlas_bvh_forest", "tlas_data", "tlas_bounding",
                "blas_meta_info", "tri_bvh_root", "tri_bvh_forest", "indices_redirect", "indices", "vertices"]


@dataclass
class BottomLevelAccelerationStructureBuildSource:
    """Triangles: positions (V,3) f32, optional u32 indices (None = non-indexed)."""

    positions: np.ndarray
    indices: np.ndarray | None = None
    flags: int = GEOMETRY_FLAG_OPAQUE


@dataclass
class TopLevelAccelerationStructureSourceInstance:
    """transform: Mat4 in the reference's element order (columns; translation at 12..14)."""

    acceleration_structure_handle: int
    transform: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32).reshape(-1))
    instance_custom_index: int = 0
    mask: int = 0xFF
    instance_shader_binding_table_record_offset: int = 0
    flags: int = 0


def _check(ctx, status: int):
    if status != native.RDN_OK:
        msg = native.lib().rdn_last_error(ctx).decode() if ctx else ""
        raise native.RdnError(status, msg)


class AccelerationStructureSystem:
    """One librdn context. device=-1 gives a host-only system (build + export, no trace)."""

    def __init__(self, device: int = 0):
        self._L = native.lib()
        h = C.c_void_p()
        st = self._L.rdn_create(C.byref(h), device)
        if st != native.RDN_OK:
            raise native.RdnError(st, f"rdn_create(device={device}) failed")
        self._h = h
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            self._L.rdn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- GPUAccelerationStructureSystemProvider ---
    def bind_tlas_max_len(self) -> int:
        return 0xFFFFFFFF

    def create_bottom_level_acceleration_structure(self, sources) -> int:
        arr = (native.Geometry * len(sources))()
        keep = []
        for g, s in zip(arr, sources):
            pos = np.ascontiguousarray(s.positions, np.float32).reshape(-1, 3)
            keep.append(pos)
            g.type = 0
            g.flags = s.flags
            g.positions = pos.ctypes.data
            g.vertex_count = pos.shape[0]
            if s.indices is not None:
                idx = np.ascontiguousarray(s.indices, np.uint32).reshape(-1)
                keep.append(idx)
                g.indices = idx.ctypes.data
                g.index_count = idx.shape[0]
        out = C.c_uint32()
        _check(self._h, self._L.rdn_blas_create(self._h, C.addressof(arr), len(sources), C.byref(out)))
        return out.value

    def delete_bottom_level_acceleration_structure(self, handle: int):
        _check(self._h, self._L.rdn_blas_delete(self._h, handle))

    def create_top_level_acceleration_structure(self, instances) -> int:
        arr = (native.Instance * len(instances))()
        for d, s in zip(arr, instances):
            tf = np.asarray(s.transform, np.float32).reshape(-1)
            for k in range(16):
                d.transform[k] = float(tf[k])
            d.custom_index = s.instance_custom_index
            d.mask = s.mask
            d.sbt_offset = s.instance_shader_binding_table_record_offset
            d.flags = s.flags
            d.blas_handle = s.acceleration_structure_handle
        out = C.c_uint32()
        _check(self._h, self._L.rdn_tlas_create(self._h, C.addressof(arr), len(instances), C.byref(out)))
        return out.value

    def delete_top_level_acceleration_structure(self, handle: int):
        _check(self._h, self._L.rdn_tlas_delete(self._h, handle))

    def bind_tlas(self, handles):
        a = np.ascontiguousarray(handles, np.uint32)
        _check(self._h, self._L.rdn_bind_tlas(self._h, a.ctypes.data, a.shape[0]))

    # --- build / inspection ---
    def build(self, blas_bin_size=0, blas_max_depth=0, tlas_bin_size=0, tlas_max_depth=0, host_threads=0,
              device_build=False):
        """device_build: build the triangle trees on the GPU (same arrays as the host build)."""
        o = native.BuildOpts(blas_bin_size, blas_max_depth, tlas_bin_size, tlas_max_depth, host_threads,
                             int(device_build))
        _check(self._h, self._L.rdn_build(self._h, C.byref(o)))

    def build_stats(self) -> dict:
        st = native.BuildStats()
        _check(self._h, self._L.rdn_get_build_stats(self._h, C.byref(st)))
        return {name: getattr(st, name) for name, _ in native.BuildStats._fields_ if name != "reserved"}

    def check_errors(self, stream=None) -> tuple[int, int]:
        """Waits for the stream and returns (status, error-word bits) of the
        kernels launched since the last check (the word is cleared)."""
        import torch

        s = (stream or torch.cuda.current_stream()).cuda_stream
        flags = C.c_uint32()
        st = self._L.rdn_check_errors(self._h, C.c_void_p(s), C.byref(flags))
        return st, flags.value

    def set_iteration_limit(self, limit: int):
        """Cap of the dynamic-fetch loops of later launches (0 = built-in)."""
        _check(self._h, self._L.rdn_set_iteration_limit(self._h, limit))

    def device_bytes(self) -> int:
        return int(self.build_stats()["device_bytes"])

    def built_array(self, name: str) -> bytes:
        which = BUILT_ARRAYS.index(name)
        size = C.c_size_t()
        _check(self._h, self._L.rdn_get_built_array(self._h, which, None, 0, C.byref(size)))
        buf = (C.c_uint8 * max(1, size.value))()
        _check(self._h, self._L.rdn_get_built_array(self._h, which, buf, size.value, C.byref(size)))
        return bytes(buf)[: size.value]

    # --- queries ---
    def _desc(self, rays, hits, hits_ext, tlas_idx, ray_flags, cull_mask, tlas_uniform, traversal, anyhit_mode,
              block_size, count=None, local_stack=0, anyhit_mask=None):
        n = rays.shape[0] if count is None else count
        return native.TraceDesc(rays.data_ptr(), hits.data_ptr(), 0 if hits_ext is None else hits_ext.data_ptr(),
                                0 if tlas_idx is None else tlas_idx.data_ptr(), n, tlas_uniform, ray_flags,
                                cull_mask, traversal, anyhit_mode, block_size, local_stack,
                                None if anyhit_mask is None else anyhit_mask.data_ptr())

    def trace(self, rays, hits, hits_ext=None, tlas_idx=None, ray_flags=0, cull_mask=0xFF, tlas_uniform=0,
              traversal=TRAVERSAL_ORDERED, anyhit_mode=ANYHIT_ACCEPT, block_size=0, stream=None, count=None,
              local_stack=0, anyhit_mask=None):
        """rays: CUDA f32 tensor (N, 8); hits: CUDA f32 tensor (N, 4) (prim id stored as u32 bits);
        hits_ext: optional CUDA int32 tensor (N, 4); tlas_idx: optional CUDA int32 tensor (N,).
        count overrides N (e.g. 0 for an empty batch). local_stack: traversal stacks in
        local memory instead of shared memory (ordered walks). anyhit_mask: CUDA int32
        bit array over built triangles (ANYHIT_PRIMITIVE_MASK)."""
        import torch

        d = self._desc(rays, hits, hits_ext, tlas_idx, ray_flags, cull_mask, tlas_uniform, traversal, anyhit_mode,
                       block_size, count, local_stack, anyhit_mask)
        s = (stream or torch.cuda.current_stream()).cuda_stream
        _check(self._h, self._L.rdn_trace(self._h, C.byref(d), C.c_void_p(s)))

    def trace_counted(self, rays, hits, hits_ext=None, tlas_idx=None, ray_flags=0, cull_mask=0xFF, tlas_uniform=0,
                      traversal=TRAVERSAL_ORDERED, anyhit_mode=ANYHIT_ACCEPT, block_size=0, stream=None) -> dict:
        import torch

        d = self._desc(rays, hits, hits_ext, tlas_idx, ray_flags, cull_mask, tlas_uniform, traversal, anyhit_mode,
                       block_size)
        s = (stream or torch.cuda.current_stream()).cuda_stream
        c = native.Counters()
        _check(self._h, self._L.rdn_trace_counted(self._h, C.byref(d), C.c_void_p(s), C.byref(c)))
        return {"node_visits": c.node_visits, "tri_tests": c.tri_tests, "tri_hits": c.tri_hits,
                "bad_tlas_rays": c.bad_tlas_rays}


PIXEL_DTYPE = np.dtype([("primary_prim", np.uint32), ("primary_t", np.float32), ("bounce_prim", np.uint32),
                        ("bounce_t", np.float32), ("primary_flags", np.uint32), ("light", np.uint32),
                        ("direct", np.float32), ("primary_instance", np.uint32)])


def camera_struct(cam) -> "native.Camera":
    """rendiation_gb300.scenes.PinholeCamera -> rdn_camera."""
    c = native.Camera()
    for name in ("origin", "forward", "right", "up"):
        v = getattr(cam, name)
        arr = getattr(c, name)
        for k in range(3):
            arr[k] = float(v[k])
    c.tan_half = float(cam.tan_half)
    c.aspect = float(cam.aspect)
    c.width = cam.width
    c.height = cam.height
    return c


class Wavefront:
    """Primary + shadow + bounce wavefront (rdn_wavefront_shadow_bounce) on one
    AccelerationStructureSystem, with its scratch queues and outputs held as
    torch CUDA tensors."""

    def __init__(self, system: AccelerationStructureSystem, camera, light, traversal=TRAVERSAL_ORDERED,
                 tlas_uniform=0, block_size=0, refill=0, rows=None):
        """rows: (row0, row1), a band of the camera's frame: the launch traces
        rows [row0, row1) with the whole frame's rays and samplers."""
        import dataclasses

        import torch

        self.system = system
        self.frame_camera = camera
        row0, row1 = rows if rows is not None else (0, camera.height)
        if not (0 <= row0 <= row1 <= camera.height):
            raise ValueError(f"band {rows} outside the frame's {camera.height} rows")
        self.rows = (row0, row1)
        camera = dataclasses.replace(camera, height=row1 - row0)
        self.camera = camera
        self.n = camera.width * camera.height
        size = C.c_size_t()
        _check(None, system._L.rdn_wavefront_scratch_size(camera.width, camera.height, C.byref(size)))
        self.scratch = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
        base = self.scratch.data_ptr()
        self.scratch_ptr = (base + 255) & ~255
        self.out = torch.empty((self.n, 8), dtype=torch.int32, device="cuda")
        self.ray_counts = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.desc = native.WavefrontDesc()
        self.desc.camera = camera_struct(camera)
        for k in range(3):
            self.desc.light[k] = float(light[k])
        self.desc.tlas_uniform = tlas_uniform
        self.desc.traversal = traversal
        self.desc.block_size = block_size
        self.desc.out = self.out.data_ptr()
        self.desc.scratch = self.scratch_ptr
        self.desc.scratch_bytes = size.value
        self.desc.ray_counts = self.ray_counts.data_ptr()
        self.desc.refill = refill
        self.desc.row_offset = row0
        self.desc.frame_height = self.frame_camera.height
        self.phase_config = None  # (primary, secondary) (traversal, block) when they differ

    def configure(self, primary, secondary, refill=None):
        """Per-kernel (traversal, block_size[, local_stack[, register_tier[,
        speculation]]]); a frame then issues one call per kernel. refill: secondary schedule (0 = batches of 32 rays
        per warp, k = dynamic fetch whenever k lanes of a warp are idle); None
        keeps the current one."""
        if refill is not None:
            self.desc.refill = refill
        primary = tuple(primary) + (0,) * (5 - len(primary))
        secondary = tuple(secondary) + (0,) * (5 - len(secondary))
        if primary == secondary:
            (self.desc.traversal, self.desc.block_size, self.desc.local_stack, self.desc.register_tier,
             self.desc.speculation) = primary
            self.phase_config = None
        else:
            self.phase_config = (primary, secondary)

    def run(self, sample_index=0, stream=None, phases=0):
        """phases: 0 both kernels, 1 primary only, 2 secondary only (queues of the last primary run)."""
        import torch

        self.desc.sample_index = sample_index
        s = (stream or torch.cuda.current_stream()).cuda_stream
        if self.phase_config is None:
            self.desc.phases = phases
            _check(self.system._h, self.system._L.rdn_wavefront_shadow_bounce(self.system._h, C.byref(self.desc),
                                                                              C.c_void_p(s)))
            return
        for ph, (trav, block, local, tier, spec) in zip((1, 2), self.phase_config):
            if phases and phases != ph:
                continue
            self.desc.phases = ph
            (self.desc.traversal, self.desc.block_size, self.desc.local_stack, self.desc.register_tier,
             self.desc.speculation) = trav, block, local, tier, spec
            _check(self.system._h, self.system._L.rdn_wavefront_shadow_bounce(self.system._h, C.byref(self.desc),
                                                                              C.c_void_p(s)))

    def results(self) -> np.ndarray:
        return self.out.cpu().numpy().view(PIXEL_DTYPE).reshape(-1)

    def rays_traced(self) -> tuple[int, int, int]:
        c = self.ray_counts.cpu().numpy()
        return int(c[0]), int(c[1]), int(c[2])


PATH_DTYPE = np.dtype([("radiance", np.float32), ("depth_flags", np.uint32)])
PATH_ESCAPED = 0x80000000
PATH_ROULETTE = 0x40000000


class Paths:
    """Batched diffuse paths (rdn_trace_paths) over rays of many scenes; each ray
    carries its index into the bound TLAS list. Buffers are torch CUDA tensors."""

    def __init__(self, system: AccelerationStructureSystem, rays, tlas_idx=None, tlas_uniform=0, max_bounces=4,
                 rr_start=2, albedo=0.5, rr_survive=0.5, seed=0, traversal=TRAVERSAL_ORDERED, block_size=0,
                 sort_key=0, refill=0):
        import torch

        self.system = system
        self.rays = rays
        self.tlas_idx = tlas_idx
        n = rays.shape[0]
        self.n = n
        self.max_bounces = max_bounces
        size = C.c_size_t()
        _check(None, system._L.rdn_paths_scratch_size(n, max_bounces, sort_key, C.byref(size)))
        self.scratch = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
        self.scratch_ptr = (self.scratch.data_ptr() + 255) & ~255
        self.out = torch.empty((max(n, 1), 2), dtype=torch.float32, device="cuda")
        self.segments_dev = torch.zeros(max_bounces + 1, dtype=torch.int32, device="cuda")
        self.desc = native.PathDesc(rays.data_ptr(), 0 if tlas_idx is None else tlas_idx.data_ptr(), n, tlas_uniform,
                                    max_bounces, rr_start, albedo, rr_survive, seed, traversal, block_size, sort_key,
                                    self.out.data_ptr(), self.scratch_ptr, size.value, self.segments_dev.data_ptr(),
                                    refill)
        self.graph = None
        self.scratch_bytes = size.value

    def configure(self, traversal=None, block_size=None, sort_key=None, refill=None, local_stack=None,
                  speculation=None):
        """Changes launch knobs (re-capture any graph afterwards). refill: 0 =
        warps trace 32 queued rays together, k = dynamic fetch whenever k lanes
        of a warp are idle."""
        import torch

        if sort_key is not None and sort_key != self.desc.sort_key:
            size = C.c_size_t()
            _check(None, self.system._L.rdn_paths_scratch_size(self.n, self.max_bounces, sort_key, C.byref(size)))
            if size.value > self.scratch_bytes:
                self.scratch = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
                self.scratch_ptr = (self.scratch.data_ptr() + 255) & ~255
                self.scratch_bytes = size.value
                self.desc.scratch = self.scratch_ptr
            self.desc.scratch_bytes = self.scratch_bytes
            self.desc.sort_key = sort_key
        if traversal is not None:
            self.desc.traversal = traversal
        if block_size is not None:
            self.desc.block_size = block_size
        if refill is not None:
            self.desc.refill = refill
        if local_stack is not None:
            self.desc.local_stack = local_stack
        if speculation is not None:
            self.desc.speculation = speculation
        self.close()

    def run(self, stream=None):
        import torch

        s = (stream or torch.cuda.current_stream()).cuda_stream
        _check(self.system._h, self.system._L.rdn_trace_paths(self.system._h, C.byref(self.desc), C.c_void_p(s)))

    def capture(self):
        """Captures the launches once into a CUDA graph (rdn_trace_paths_graph)."""
        g = C.c_void_p()
        _check(self.system._h, self.system._L.rdn_trace_paths_graph(self.system._h, C.byref(self.desc), C.byref(g)))
        self.graph = g

    def launch_graph(self, stream=None):
        import torch

        s = (stream or torch.cuda.current_stream()).cuda_stream
        st = self.system._L.rdn_graph_launch(self.graph, C.c_void_p(s))
        if st != native.RDN_OK:
            raise native.RdnError(st, "rdn_graph_launch failed")

    def close(self):
        if self.graph:
            self.system._L.rdn_graph_destroy(self.graph)
            self.graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def results(self) -> np.ndarray:
        return self.out.cpu().numpy()[: self.n].view(PATH_DTYPE).reshape(-1)

    def segments(self) -> list[int]:
        return [int(x) for x in self.segments_dev.cpu().numpy()]


def hits_to_numpy(hits) -> np.ndarray:
    """(N,4) f32 CUDA tensor -> structured array (t, u, v, prim)."""
    h = hits.detach().cpu().numpy().astype(np.float32, copy=False)
    out = np.zeros(h.shape[0], dtype=[("t", np.float32), ("u", np.float32), ("v", np.float32), ("prim", np.uint32)])
    out["t"], out["u"], out["v"] = h[:, 0], h[:, 1], h[:, 2]
    out["prim"] = h[:, 3].view(np.uint32)
    return out
