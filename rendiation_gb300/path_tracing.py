"""The reference path tracer on an acceleration-structure system.

Mirrors ``DeviceReferencePathTracingRenderer``
(scene/rendering/gpu-ray-tracing/src/feature/path_tracing/mod.rs:82-235):
``render`` adds one sample per pixel to an RGBA8 unorm buffer (the
reference's radiance texture, frame_state.rs:12-20) and advances the sample
count (``PTRenderState::next_sample``); ``reset_sample`` restarts the average.
The frame is one fused CUDA kernel (librdn ``rdn_path_tracing_render``):
camera ray, closest hit with light sampling and its shadow ray, BRDF
importance sampling, miss, tone map and running average.

Scene inputs follow the reference's scene bridge: directional lights
(DirectionalLightStorage: illuminance, direction; path_tracing/lighting_bridge.rs:213-258),
physical materials by instance custom index (the channels of
PhysicalShading::construct_shading_impl, direct_lighting.rs:14-59), optional
per-vertex shading normals, a solid or test background (ray_miss.rs:30-152)
and a tone map (content/texture/gpu-process/src/tonemap.rs).
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import native
from .raytracing import TRAVERSAL_ORDERED_WIDE, _check

TONE_MAP_NONE, TONE_MAP_LINEAR, TONE_MAP_REINHARD, TONE_MAP_CINEON, TONE_MAP_ACES_FILMIC = 0, 1, 2, 3, 4
BACKGROUND_SOLID, BACKGROUND_TEST, BACKGROUND_ENV_CUBE = 0, 1, 2
SCHEDULE_PIXEL, SCHEDULE_REFILL, SCHEDULE_WAVEFRONT = 0, 1, 2
MAX_RAY_DEPTH = 3  # path_tracing/mod.rs:80

MATERIAL_DTYPE = np.dtype([("base_color", np.float32, 3), ("perceptual_roughness", np.float32),
                           ("emissive", np.float32, 3), ("metallic", np.float32), ("specular", np.float32, 3),
                           ("reflectance", np.float32), ("workflow", np.uint32), ("reserved", np.uint32, 3)])
DIRECTIONAL_LIGHT_DTYPE = np.dtype([("illuminance", np.float32, 3), ("direction", np.float32, 3)])
assert MATERIAL_DTYPE.itemsize == 64 and DIRECTIONAL_LIGHT_DTYPE.itemsize == 24


def clamp_size_by_area(width: int, height: int, area: int = 512 * 512) -> tuple[int, int]:
    """The render size the reference path tracer uses for a frame
    (gpu-ray-tracing/src/lib.rs:44-53: scale both sides by sqrt(area / w h) in
    f32, floor, at least 1)."""
    assert area >= 1
    ratio = np.float32(area) / np.float32(width * height)
    ratio = np.float32(math.sqrt(ratio))
    w = int(math.floor(np.float32(width) * ratio))
    h = int(math.floor(np.float32(height) * ratio))
    return max(w, 1), max(h, 1)


def metallic_material(base_color=(0.5, 0.5, 0.5), roughness=0.5, metallic=0.0, reflectance=0.5, emissive=(0, 0, 0)):
    m = np.zeros((), MATERIAL_DTYPE)
    m["base_color"], m["perceptual_roughness"], m["metallic"] = base_color, roughness, metallic
    m["reflectance"], m["emissive"], m["workflow"] = reflectance, emissive, 0
    return m


def specular_material(base_color=(0.5, 0.5, 0.5), roughness=0.5, specular=(0.04, 0.04, 0.04), emissive=(0, 0, 0)):
    m = np.zeros((), MATERIAL_DTYPE)
    m["base_color"], m["perceptual_roughness"], m["specular"] = base_color, roughness, specular
    m["emissive"], m["workflow"] = emissive, 1
    return m


def directional_light(illuminance, direction):
    d = np.asarray(direction, np.float64)
    l = np.zeros((), DIRECTIONAL_LIGHT_DTYPE)
    l["illuminance"], l["direction"] = illuminance, (d / np.linalg.norm(d)).astype(np.float32)
    return l


def _stream(stream):
    import torch

    return C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)


class DeviceReferencePathTracingRenderer:
    """One path-traced sample per ``render`` call into ``image`` (RGBA8,
    width*height*4 bytes). ``lights``, ``materials`` and ``sm_to_material``
    are numpy arrays (DIRECTIONAL_LIGHT_DTYPE, MATERIAL_DTYPE, uint32) copied to
    the device once; ``normals`` is a CUDA float tensor of 3 per built vertex
    or None. With ``keep_radiance`` the last sample's HDR radiance and path
    length per pixel are kept in ``radiance`` (float32, width*height*4).
    ``speculation`` is the ordered walks' leaf postponement threshold (a lane
    holding a leaf keeps descending while more than this many lanes of its
    warp still look for one)."""

    def __init__(self, system, width, height, view_projection_inv, camera_position, lights=None, materials=None,
                 sm_to_material=None, normals=None, max_path_depth=MAX_RAY_DEPTH, tone_map=TONE_MAP_ACES_FILMIC,
                 exposure=1.0, background=BACKGROUND_SOLID, background_color=(0.0, 0.0, 0.0),
                 traversal=TRAVERSAL_ORDERED_WIDE, tlas_uniform=0, block_size=0, keep_radiance=False,
                 count_rays=False, schedule=SCHEDULE_REFILL, register_tier=0, env_cube=None, env_transform=None,
                 env_intensity=1.0, speculation=0):
        import torch

        self.system = system
        self.width, self.height = int(width), int(height)
        self.image = torch.zeros(self.width * self.height * 4, dtype=torch.uint8, device="cuda")
        self.vp_inv = np.asarray(view_projection_inv, np.float32).reshape(16)
        self.cam = np.asarray(camera_position, np.float32).reshape(3)
        if lights is None or len(lights) == 0:
            lights = np.zeros(0, DIRECTIONAL_LIGHT_DTYPE)
        lights = np.asarray(lights, DIRECTIONAL_LIGHT_DTYPE).reshape(-1)
        self.light_count = len(lights)
        self._lights = (torch.from_numpy(lights.view(np.uint8).copy()).cuda() if len(lights) else None)
        self.material_count = 0
        self._materials = None
        if materials is not None:
            mats = np.asarray(materials, MATERIAL_DTYPE).reshape(-1)
            self.material_count = len(mats)
            self._materials = torch.from_numpy(mats.view(np.uint8).copy()).cuda() if len(mats) else None
        self._sm = None
        self.sm_count = 0
        if sm_to_material is not None:
            sm = np.asarray(sm_to_material, np.uint32).reshape(-1)
            self.sm_count = len(sm)
            # an empty table is a non-null table of length 0: every instance takes the default material
            self._sm = torch.from_numpy(sm.view(np.int32).copy() if len(sm) else np.zeros(1, np.int32)).cuda()
        self.normals = normals
        self.max_path_depth = max_path_depth
        self.tone_map, self.exposure = tone_map, exposure
        self.background, self.background_color = background, tuple(float(c) for c in background_color)
        self.traversal, self.tlas_uniform, self.block_size = traversal, tlas_uniform, block_size
        self.schedule = schedule
        self.register_tier = register_tier
        self.speculation = speculation
        # environment cube (BACKGROUND_ENV_CUBE): float32 (6, size, size, 4), faces +X -X +Y -Y +Z -Z
        self._env = None
        self.env_size = 0
        if env_cube is not None:
            cube = np.ascontiguousarray(env_cube, np.float32)
            assert cube.ndim == 4 and cube.shape[0] == 6 and cube.shape[1] == cube.shape[2] and cube.shape[3] == 4
            self.env_size = cube.shape[1]
            self._env = torch.from_numpy(cube.reshape(-1).copy()).cuda()
        self.env_transform = np.asarray(env_transform if env_transform is not None else np.eye(4), np.float32)
        self.env_intensity = float(env_intensity)
        self.radiance = (torch.zeros(self.width * self.height * 4, dtype=torch.float32, device="cuda")
                         if keep_radiance else None)
        self.ray_counts = torch.zeros(2, dtype=torch.int32, device="cuda") if count_rays else None
        self.sample_count = 0
        self._scratch = None

    def _scratch_ptr(self):
        """Path state and queues of the wavefront schedule (allocated on first use)."""
        if self._scratch is None:
            import torch

            size = C.c_size_t()
            _check(self.system._h, self.system._L.rdn_pt_scratch_size(self.width, self.height, C.byref(size)))
            self._scratch = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
            self._scratch_bytes = size.value
        return (self._scratch.data_ptr() + 255) & ~255, self._scratch_bytes

    def desc(self) -> native.PtDesc:
        d = native.PtDesc()
        d.view_projection_inv[:] = [float(v) for v in self.vp_inv]
        d.camera_position[:] = [float(v) for v in self.cam]
        d.width, d.height, d.sample_count = self.width, self.height, self.sample_count
        d.max_path_depth, d.tlas_uniform, d.traversal = self.max_path_depth, self.tlas_uniform, self.traversal
        d.tone_map, d.exposure, d.background = self.tone_map, self.exposure, self.background
        d.background_color[:] = self.background_color
        d.lights = self._lights.data_ptr() if self._lights is not None else None
        d.light_count = self.light_count
        d.materials = self._materials.data_ptr() if self._materials is not None else None
        d.material_count = self.material_count
        d.sm_to_material = self._sm.data_ptr() if self._sm is not None else None
        d.sm_count = self.sm_count
        d.block_size = self.block_size
        d.normals = self.normals.data_ptr() if self.normals is not None else None
        d.image = self.image.data_ptr()
        d.radiance = self.radiance.data_ptr() if self.radiance is not None else None
        d.ray_counts = self.ray_counts.data_ptr() if self.ray_counts is not None else None
        d.schedule = self.schedule
        d.register_tier = self.register_tier
        d.speculation = self.speculation
        d.env_cube = self._env.data_ptr() if self._env is not None else None
        d.env_size = self.env_size
        d.env_transform[:] = [float(v) for v in self.env_transform.T.reshape(-1)]  # columns, reference order
        d.env_intensity = self.env_intensity
        if self.schedule == SCHEDULE_WAVEFRONT:
            d.scratch, d.scratch_bytes = self._scratch_ptr()
        return d

    def capture(self, counter):
        """One sample captured into a CUDA graph (rdn_pt_capture) that reads its
        sample index from `counter` (a CUDA int32 tensor of one element) and
        advances it; returns a callable that replays the sample."""
        d = self.desc()
        d.sample_counter = counter.data_ptr()
        g = C.c_void_p()
        _check(self.system._h, self.system._L.rdn_pt_capture(self.system._h, C.byref(d), C.byref(g)))
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
        _check(self.system._h, self.system._L.rdn_path_tracing_render(self.system._h, C.byref(d), _stream(stream)))
        self.sample_count += 1

    def reset_sample(self):
        self.sample_count = 0
        self.image.zero_()

    def result(self) -> np.ndarray:
        return self.image.cpu().numpy().reshape(self.height, self.width, 4)

    def rays_traced(self) -> tuple[int, int]:
        """(core, shadow) rays traced since creation (count_rays=True)."""
        c = self.ray_counts.cpu().numpy().view(np.uint32)
        return int(c[0]), int(c[1])
