"""ctypes wrapper of the oracle library (oracle/_build/liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and bench.py's
CPU-baseline / reference arm, as the checker. The product never imports it.
The oracle is a C++ restatement of the reference's CPU ray-query path
(see rdn_oracle.cpp for the file:line map); parity with the reference's own
outputs is unpinned because the Rust reference cannot be built here.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lib = None

HIT_DTYPE = np.dtype(
    [("t", np.float32), ("u", np.float32), ("v", np.float32), ("prim", np.uint32),
     ("geometry", np.uint32), ("instance", np.uint32), ("custom", np.uint32), ("hit_kind", np.uint32)]
)
MISS = 0xFFFFFFFF
RAY_DTYPE = np.dtype([("org", np.float32, 3), ("tmin", np.float32), ("dir", np.float32, 3), ("tmax", np.float32)])

BUF_TLAS_BINDING, BUF_TLAS_BVH_ROOT, BUF_TLAS_BVH_FOREST, BUF_TLAS_DATA, BUF_TLAS_BOUNDING = 0, 1, 2, 3, 4
BUF_BLAS_META_INFO, BUF_TRI_BVH_ROOT, BUF_TRI_BVH_FOREST, BUF_INDICES_REDIRECT, BUF_INDICES, BUF_VERTICES = 5, 6, 7, 8, 9, 10


# rdn_pt_material / rdn_pt_directional_light layouts (64 B / 24 B)
PT_MATERIAL_DTYPE = np.dtype([("base_color", np.float32, 3), ("perceptual_roughness", np.float32),
                              ("emissive", np.float32, 3), ("metallic", np.float32), ("specular", np.float32, 3),
                              ("reflectance", np.float32), ("workflow", np.uint32), ("reserved", np.uint32, 3)])
PT_LIGHT_DTYPE = np.dtype([("illuminance", np.float32, 3), ("direction", np.float32, 3)])


class _PtScene(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("tone_map", C.c_uint32), ("background", C.c_uint32),
                ("exposure", C.c_float), ("bg", C.c_float * 3), ("lights", C.c_void_p), ("light_count", C.c_uint32),
                ("materials", C.c_void_p), ("material_count", C.c_uint32), ("sm_to_material", C.c_void_p),
                ("sm_count", C.c_uint32), ("env", C.c_void_p), ("env_size", C.c_uint32),
                ("env_transform", C.c_float * 16), ("env_intensity", C.c_float)]


def _pt_scene(lights, materials, sm_to_material, max_depth, tone_map, exposure, background, bg, env_cube=None,
              env_transform=None, env_intensity=1.0):
    sc = _PtScene()
    sc.max_depth, sc.tone_map, sc.background, sc.exposure = max_depth, tone_map, background, exposure
    sc.bg[:] = [float(b) for b in bg]
    keep = []
    if env_cube is not None:
        cube = np.ascontiguousarray(env_cube, np.float32)
        keep.append(cube)
        sc.env, sc.env_size = cube.ctypes.data, cube.shape[1]
    m = np.asarray(env_transform if env_transform is not None else np.eye(4), np.float32)
    sc.env_transform[:] = [float(v) for v in m.T.reshape(-1)]  # columns, the reference's memory order
    sc.env_intensity = env_intensity
    if lights is not None and len(lights):
        la = np.ascontiguousarray(lights, PT_LIGHT_DTYPE)
        keep.append(la)
        sc.lights, sc.light_count = la.ctypes.data, len(la)
    if materials is not None and len(materials):
        ma = np.ascontiguousarray(materials, PT_MATERIAL_DTYPE)
        keep.append(ma)
        sc.materials, sc.material_count = ma.ctypes.data, len(ma)
    if sm_to_material is not None:
        sa = np.ascontiguousarray(sm_to_material, np.uint32)
        keep.append(sa)
        sc.sm_to_material, sc.sm_count = (sa.ctypes.data if len(sa) else None), len(sa)
        if not len(sa):  # an empty table still routes every custom index to the default material
            keep.append(np.zeros(1, np.uint32))
            sc.sm_to_material = keep[-1].ctypes.data
    return sc, keep


def pt_surface_query(seed, view, normal, l2, materials=None, sm_to_material=None, sm_id=0):
    """Oracle PT surface for tests: (direction, bsdf, pdf) of the BRDF sample
    drawn from PCG state `seed`, (bsdf, pdf) at direction l2, and
    (albedo, f0, alpha, estimate) of the surface."""
    sc, keep = _pt_scene(None, materials, sm_to_material, 0, 0, 1.0, 0, (0, 0, 0))
    o1, o2, o3 = np.zeros(7, np.float32), np.zeros(4, np.float32), np.zeros(8, np.float32)
    v, n, l = (np.ascontiguousarray(a, np.float32) for a in (view, normal, l2))
    lib().orc_pt_surface_query(C.byref(sc), sm_id, _ptr(v), _ptr(n), seed, _ptr(l), _ptr(o1), _ptr(o2), _ptr(o3))
    return (o1[:3], o1[3:6], float(o1[6])), (o2[:3], float(o2[3])), (o3[:3], o3[3:6], float(o3[6]), float(o3[7]))


def pt_math(op: str, x, arg=0) -> np.ndarray:
    """The oracle's fixed-polynomial functions: atan, log2, exp2, pow22, tone (x channel of tone map `arg`)."""
    code = {"atan": 0, "log2": 1, "exp2": 2, "pow22": 3, "tone": 4}[op]
    xa = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(xa)
    lib().orc_pt_math(code, arg, _ptr(xa), _ptr(y), xa.size)
    return y


class _Geometry(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("vertex_count", C.c_uint32), ("indices", C.c_void_p),
                ("index_count", C.c_uint32), ("flags", C.c_uint32), ("type", C.c_uint32)]


class _Instance(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("custom_index", C.c_uint32), ("mask", C.c_uint32),
                ("sbt_offset", C.c_uint32), ("flags", C.c_uint32), ("blas_handle", C.c_uint32)]


def build_library() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build_library()
        L = C.CDLL(_LIB_PATH)
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        L.orc_create.restype = vp
        L.orc_destroy.argtypes = [vp]
        L.orc_last_error.restype = C.c_char_p
        L.orc_last_error.argtypes = [vp]
        L.orc_blas_create.argtypes = [vp, vp, u32, C.POINTER(u32)]
        L.orc_blas_delete.argtypes = [vp, u32]
        L.orc_tlas_create.argtypes = [vp, vp, u32, C.POINTER(u32)]
        L.orc_tlas_delete.argtypes = [vp, u32]
        L.orc_bind_tlas.argtypes = [vp, vp, u32]
        L.orc_build.argtypes = [vp, u32, u32, u32, u32]
        L.orc_build_stats.argtypes = [vp, vp]
        L.orc_get_buffer.restype = C.c_size_t
        L.orc_get_buffer.argtypes = [vp, i32, vp, C.c_size_t]
        L.orc_trace.argtypes = [vp, vp, u32, vp, u32, u32, u32, u32, vp, vp, vp, vp, i32, C.POINTER(C.c_double), i32]
        L.orc_nan_exposure.argtypes = [vp, vp, u32, vp, u32, u32, u32, vp, i32]
        L.orc_eval_fp64.argtypes = [vp, vp, u32, vp, vp]
        L.orc_edge_margin.argtypes = [vp, vp, u32, vp, vp]
        L.orc_bruteforce_fp64.argtypes = [vp, vp, u32, u32, vp, i32]
        L.orc_intersect_triangle.argtypes = [vp, vp, C.c_float, C.c_float, vp, vp, vp, i32, i32, vp]
        L.orc_intersect_aabb.argtypes = [vp, vp, C.c_float, C.c_float, vp, vp]
        L.orc_select_nth.argtypes = [vp, vp, C.c_size_t, C.c_size_t]
        L.orc_trace_paths.argtypes = [vp, vp, u32, vp, u32, u32, u32, C.c_float, C.c_float, u32, vp, vp, i32,
                                      C.POINTER(C.c_double)]
        L.orc_path_segments.argtypes = [vp, vp, u32, vp, u32, u32, u32, vp, vp, i32]
        L.orc_ao_render.argtypes = [vp, vp, vp, u32, u32, u32, u32, vp, vp, u32, u32, i32, vp,
                                    C.POINTER(C.c_double)]
        L.orc_wavefront_shadow_bounce.argtypes = [vp, vp, u32, u32, vp, u32, u32, u32, u32, vp, vp, i32,
                                                  C.POINTER(C.c_double), i32]
        L.orc_wavefront_pixel_rays.argtypes = [vp, vp, u32, u32, vp, u32, u32, vp, u32, vp, vp, i32, i32]
        L.orc_pt_render.argtypes = [vp, vp, vp, u32, u32, u32, u32, vp, vp, vp, vp, u32, u32, i32, i32, vp,
                                    C.POINTER(C.c_double)]
        L.orc_pt_surface_query.argtypes = [vp, u32, vp, vp, u32, vp, vp, vp, vp]
        L.orc_pt_math.argtypes = [i32, u32, vp, vp, C.c_uint64]
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


class OracleSystem:
    """Mirror of the reference's NaiveSahBVHSystem (naive/mod.rs:496-609) on the CPU."""

    def __init__(self):
        self._L = lib()
        self._h = self._L.orc_create()
        self._keep = []

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.orc_destroy(self._h)
            self._h = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle error {rc}: {self._L.orc_last_error(self._h).decode()}")

    def create_blas(self, geometries) -> int:
        """geometries: list of (positions (V,3) f32, indices u32 or None, flags)."""
        arr = (_Geometry * len(geometries))()
        keep = []
        for g, (pos, idx, flags) in zip(arr, geometries):
            pos = np.ascontiguousarray(pos, np.float32)
            keep.append(pos)
            g.positions = pos.ctypes.data
            g.vertex_count = pos.shape[0]
            if idx is not None:
                idx = np.ascontiguousarray(idx, np.uint32)
                keep.append(idx)
                g.indices = idx.ctypes.data
                g.index_count = idx.shape[0]
            g.flags = flags
            g.type = 0
        out = C.c_uint32()
        self._check(self._L.orc_blas_create(self._h, C.addressof(arr), len(geometries), C.byref(out)))
        return out.value

    def delete_blas(self, h: int):
        self._check(self._L.orc_blas_delete(self._h, h))

    def create_tlas(self, instances) -> int:
        """instances: list of dicts with transform (4x4, column-major flat 16), blas, custom, mask, sbt, flags."""
        arr = (_Instance * len(instances))()
        for dst, s in zip(arr, instances):
            tf = np.asarray(s.get("transform", np.eye(4, dtype=np.float32).reshape(-1)), np.float32).reshape(-1)
            for k in range(16):
                dst.transform[k] = float(tf[k])
            dst.custom_index = s.get("custom", 0)
            dst.mask = s.get("mask", 0xFF)
            dst.sbt_offset = s.get("sbt", 0)
            dst.flags = s.get("flags", 0)
            dst.blas_handle = s["blas"]
        out = C.c_uint32()
        self._check(self._L.orc_tlas_create(self._h, C.addressof(arr), len(instances), C.byref(out)))
        return out.value

    def delete_tlas(self, h: int):
        self._check(self._L.orc_tlas_delete(self._h, h))

    def bind_tlas(self, handles):
        a = np.ascontiguousarray(handles, np.uint32)
        self._check(self._L.orc_bind_tlas(self._h, _ptr(a), a.shape[0]))

    def build(self, blas_bin_size=2, blas_max_depth=50, tlas_bin_size=10, tlas_max_depth=50):
        self._check(self._L.orc_build(self._h, blas_bin_size, blas_max_depth, tlas_bin_size, tlas_max_depth))

    def build_stats(self):
        s = np.zeros(2, np.uint64)
        self._check(self._L.orc_build_stats(self._h, _ptr(s)))
        return {"sah_splits": int(s[0]), "median_fallbacks": int(s[1])}

    def buffer(self, which: int) -> bytes:
        n = self._L.orc_get_buffer(self._h, which, None, 0)
        b = np.zeros(n, np.uint8)
        self._L.orc_get_buffer(self._h, which, _ptr(b), n)
        return b.tobytes()

    def trace(self, rays: np.ndarray, tlas_idx=None, tlas_uniform=0, ray_flags=0, cull_mask=0xFF, anyhit_mode=0,
              threads=1, counts=False, anyhit_mask=None, watertight=False):
        """anyhit_mask: uint32 bit array over built triangles (anyhit_mode 3).
        watertight: the watertight triangle test instead of the reference's."""
        rays = np.ascontiguousarray(rays)
        n = rays.shape[0]
        out = np.zeros(n, HIT_DTYPE)
        rc = np.zeros((n, 2), np.uint32) if counts else None
        tot = np.zeros(6, np.uint64)
        ti = None if tlas_idx is None else np.ascontiguousarray(tlas_idx, np.uint32)
        sec = C.c_double()
        mask = None if anyhit_mask is None else np.ascontiguousarray(anyhit_mask, np.uint32)
        self._check(self._L.orc_trace(self._h, _ptr(rays), n, _ptr(ti), tlas_uniform, ray_flags, cull_mask,
                                      anyhit_mode, _ptr(mask), _ptr(out), _ptr(rc), _ptr(tot), threads,
                                      C.byref(sec), 1 if watertight else 0))
        totals = dict(zip(["tri_visit", "tri_hit", "bvh_visit", "bvh_hit", "far_assert", "bad_tlas"],
                          (int(x) for x in tot)))
        totals["seconds"] = sec.value
        if counts:
            return out, totals, rc
        return out, totals

    def nan_exposure(self, rays: np.ndarray, tlas_idx=None, tlas_uniform=0, ray_flags=0, cull_mask=0xFF,
                     threads=4) -> np.ndarray:
        """Per ray: True when some triangle its boxes admit (far held at tmax) gives a NaN
        distance, so that the result depends on the order of the walk."""
        rays = np.ascontiguousarray(rays)
        out = np.zeros(rays.shape[0], np.uint8)
        ti = None if tlas_idx is None else np.ascontiguousarray(tlas_idx, np.uint32)
        self._check(self._L.orc_nan_exposure(self._h, _ptr(rays), rays.shape[0], _ptr(ti), tlas_uniform, ray_flags,
                                             cull_mask, _ptr(out), threads))
        return out.astype(bool)

    def eval_fp64(self, rays: np.ndarray, hits: np.ndarray) -> np.ndarray:
        out = np.zeros((rays.shape[0], 3), np.float64)
        self._check(self._L.orc_eval_fp64(self._h, _ptr(np.ascontiguousarray(rays)), rays.shape[0],
                                          _ptr(np.ascontiguousarray(hits)), _ptr(out)))
        return out

    def edge_margin(self, rays: np.ndarray, hits: np.ndarray) -> np.ndarray:
        """Per hit: [FP64 distance of the ray's plane point to the triangle's
        nearest edge (negative outside), f32 position error bound of the
        reference's formula]; NaN for misses."""
        out = np.zeros((rays.shape[0], 2), np.float64)
        self._check(self._L.orc_edge_margin(self._h, _ptr(np.ascontiguousarray(rays)), rays.shape[0],
                                            _ptr(np.ascontiguousarray(hits)), _ptr(out)))
        return out

    def bruteforce_fp64(self, rays: np.ndarray, tlas_uniform=0, threads=4) -> np.ndarray:
        out = np.zeros((rays.shape[0], 5), np.float64)
        self._check(self._L.orc_bruteforce_fp64(self._h, _ptr(np.ascontiguousarray(rays)), rays.shape[0],
                                                tlas_uniform, _ptr(out), threads))
        return out


PIXEL_DTYPE = np.dtype([("primary_prim", np.uint32), ("primary_t", np.float32), ("bounce_prim", np.uint32),
                        ("bounce_t", np.float32), ("primary_flags", np.uint32), ("light", np.uint32),
                        ("direct", np.float32), ("primary_instance", np.uint32)])


def wavefront_shadow_bounce(system: OracleSystem, cam_floats, width, height, light, sample_index=0, tlas=0,
                            row0=0, row1=None, threads=1, watertight=False):
    """The oracle's primary + shadow + bounce pipeline over rows [row0, row1).
    Returns (pixel records, [primary, shadow, bounce] rays, seconds)."""
    row1 = height if row1 is None else row1
    cam = np.ascontiguousarray(cam_floats, np.float32)
    li = np.ascontiguousarray(light, np.float32)
    out = np.zeros((row1 - row0) * width, PIXEL_DTYPE)
    rays = np.zeros(3, np.uint64)
    sec = C.c_double()
    system._check(system._L.orc_wavefront_shadow_bounce(system._h, _ptr(cam), width, height, _ptr(li), sample_index,
                                                        tlas, row0, row1, _ptr(out), _ptr(rays), threads,
                                                        C.byref(sec), 1 if watertight else 0))
    return out, [int(x) for x in rays], sec.value


def wavefront_pixel_rays(system: OracleSystem, cam_floats, width, height, light, pixels, sample_index=0, tlas=0,
                         threads=1, watertight=False):
    """The oracle's primary, shadow and bounce rays of the given pixels (y * width + x).
    Returns (primary rays, shadow rays, bounce rays, primary-hit flags); the
    shadow and bounce rays of a pixel whose primary missed are zero."""
    pixels = np.ascontiguousarray(pixels, np.uint32)
    n = pixels.shape[0]
    rays = np.zeros(3 * max(n, 1), RAY_DTYPE)
    has = np.zeros(max(n, 1), np.uint8)
    cam = np.ascontiguousarray(cam_floats, np.float32)
    li = np.ascontiguousarray(light, np.float32)
    system._check(system._L.orc_wavefront_pixel_rays(system._h, _ptr(cam), width, height, _ptr(li), sample_index,
                                                     tlas, _ptr(pixels), n, _ptr(rays), _ptr(has), threads,
                                                     1 if watertight else 0))
    return (rays[0:3 * n:3].copy(), rays[1:3 * n:3].copy(), rays[2:3 * n:3].copy(), has[:n].astype(bool))


PATH_DTYPE = np.dtype([("radiance", np.float32), ("depth_flags", np.uint32)])


def trace_paths(system: OracleSystem, rays, tlas_idx=None, tlas_uniform=0, max_bounces=4, rr_start=2, albedo=0.5,
                rr_survive=0.5, seed=0, threads=1):
    """The oracle's batched diffuse paths. Returns (results, rays per bounce, seconds)."""
    rays = np.ascontiguousarray(rays)
    n = rays.shape[0]
    out = np.zeros(n, PATH_DTYPE)
    seg = np.zeros(max_bounces + 1, np.uint64)
    ti = None if tlas_idx is None else np.ascontiguousarray(tlas_idx, np.uint32)
    sec = C.c_double()
    system._check(system._L.orc_trace_paths(system._h, _ptr(rays), n, _ptr(ti), tlas_uniform, max_bounces, rr_start,
                                            albedo, rr_survive, seed, _ptr(out), _ptr(seg), threads, C.byref(sec)))
    return out, [int(x) for x in seg], sec.value


def path_segments(system: OracleSystem, rays, tlas_idx=None, tlas_uniform=0, segments=3, seed=0, threads=1):
    """Per-segment rays and hit triangles of differentiable paths (seg_tri ~0 = miss)."""
    rays = np.ascontiguousarray(rays)
    n = rays.shape[0]
    seg_rays = np.zeros(n * segments, rays.dtype)
    seg_tri = np.zeros(n * segments, np.uint32)
    ti = None if tlas_idx is None else np.ascontiguousarray(tlas_idx, np.uint32)
    system._check(system._L.orc_path_segments(system._h, _ptr(rays), n, _ptr(ti), tlas_uniform, segments, seed,
                                              _ptr(seg_rays), _ptr(seg_tri), threads))
    return seg_rays, seg_tri


def intersect_triangle(o, d, near, far, v0, v1, v2, cull_enable=False, cull_back=False):
    f = lambda a: np.ascontiguousarray(a, np.float32)
    o, d, v0, v1, v2 = f(o), f(d), f(v0), f(v1), f(v2)
    out = np.zeros(4, np.float32)
    lib().orc_intersect_triangle(_ptr(o), _ptr(d), near, far, _ptr(v0), _ptr(v1), _ptr(v2), int(cull_enable),
                                 int(cull_back), _ptr(out))
    return out


def intersect_aabb(o, d, tmin, tmax, bmin, bmax) -> bool:
    f = lambda a: np.ascontiguousarray(a, np.float32)
    o, d, bmin, bmax = f(o), f(d), f(bmin), f(bmax)
    return bool(lib().orc_intersect_aabb(_ptr(o), _ptr(d), tmin, tmax, _ptr(bmin), _ptr(bmax)))


def select_nth(keys: np.ndarray, index: int) -> np.ndarray:
    keys = np.ascontiguousarray(keys, np.float32)
    idx = np.arange(keys.shape[0], dtype=np.uint64)
    lib().orc_select_nth(_ptr(keys), _ptr(idx), keys.shape[0], index)
    return idx


def pt_render(system: OracleSystem, vp_inv, cam, width, height, image: np.ndarray, lights=None, materials=None,
              sm_to_material=None, max_depth=3, tone_map=4, exposure=1.0, background=0, bg=(0.0, 0.0, 0.0),
              sample_count=0, tlas=0, normals=None, rows=None, radiance: np.ndarray | None = None, intersector=0,
              threads=4, env_cube=None, env_transform=None, env_intensity=1.0):
    """One path-tracing sample into image (uint32 RGBA8 texels, width*height,
    updated in place) for rows [r0, r1); radiance (float32 width*height*4,
    optional) receives the sample's HDR radiance and core-ray count per pixel.
    Returns ((core, shadow) rays traced, seconds)."""
    vp = np.ascontiguousarray(vp_inv, np.float32)
    cm = np.ascontiguousarray(cam, np.float32)
    assert image.dtype == np.uint32 and image.size == width * height and image.flags.c_contiguous
    if radiance is not None:
        assert radiance.dtype == np.float32 and radiance.size == 4 * width * height and radiance.flags.c_contiguous
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    sc, keep = _pt_scene(lights, materials, sm_to_material, max_depth, tone_map, exposure, background, bg,
                         env_cube, env_transform, env_intensity)
    r0, r1 = rows if rows is not None else (0, height)
    rays = np.zeros(2, np.uint64)
    sec = C.c_double()
    rc = lib().orc_pt_render(system._h, _ptr(vp), _ptr(cm), width, height, sample_count, tlas, _ptr(nrm),
                             C.byref(sc), _ptr(image), _ptr(radiance), r0, r1, intersector, threads, _ptr(rays),
                             C.byref(sec))
    system._check(rc)
    del keep
    return (int(rays[0]), int(rays[1])), sec.value


def ao_render(system: OracleSystem, vp_inv, cam, width, height, image: np.ndarray, sample_count=0, tlas=0,
              normals=None, rows=None, threads=4):
    """One AO sample into image (uint32 RGBA8 texels, width*height, updated in
    place) for rows [r0, r1). Returns (rays traced [camera, occlusion], seconds)."""
    vp = np.ascontiguousarray(vp_inv, np.float32)
    cm = np.ascontiguousarray(cam, np.float32)
    assert image.dtype == np.uint32 and image.size == width * height and image.flags.c_contiguous
    nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
    r0, r1 = rows if rows is not None else (0, height)
    rays = np.zeros(2, np.uint64)
    sec = C.c_double()
    rc = lib().orc_ao_render(system._h, _ptr(vp), _ptr(cm), width, height, sample_count, tlas, _ptr(nrm), _ptr(image),
                             r0, r1, threads, _ptr(rays), C.byref(sec))
    system._check(rc)
    return (int(rays[0]), int(rays[1])), sec.value
