"""Seeded synthetic scenes and ray sets for the ray-query workloads.

Every generator is deterministic for a given seed: random numbers come from
numpy's PCG64 bit generator (``np.random.Generator(np.random.PCG64(seed))``),
positions are computed in float64 and rounded once to float32, and ray
directions are computed with float32 arithmetic in a fixed operation order.

Workloads (sizes are the defaults of each function):

* ``triangle_soup`` — N triangles, each centroid uniform in [0,1]^3 and each
  of the three vertex offsets uniform in [-0.02, 0.02]^3, non-indexed.
* ``heightfield`` — an n x n vertex grid over [0,1]^2 with
  z = sum_{k in 2,4,8,16} (0.1/k) sin(2 pi k (x cos th_k + y sin th_k) + ph_k),
  th, ph uniform in [0, 2 pi) per octave; 2 (n-1)^2 indexed triangles.
* ``pinhole_rays`` — one primary ray per pixel centre of a pinhole camera.
* ``sphere_rays`` — origins uniform in a box, directions uniform on S^2.

The reference's fixtures use the same ray convention for pixel centres
(shader/ray-tracing/src/backend/wavefront_compute/geometry/naive/test.rs:259-266).
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

F32 = np.float32


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


@dataclass
class Mesh:
    positions: np.ndarray  # (V, 3) float32
    indices: np.ndarray | None  # (T*3,) uint32 or None (non-indexed)

    @property
    def triangle_count(self) -> int:
        if self.indices is None:
            return self.positions.shape[0] // 3
        return self.indices.shape[0] // 3

    def triangles(self) -> np.ndarray:
        """(T, 3, 3) float32 vertex positions per triangle."""
        if self.indices is None:
            return self.positions.reshape(-1, 3, 3)
        return self.positions[self.indices.reshape(-1, 3)]


def triangle_soup(n_tris: int = 10_000, seed: int = 0, offset: float = 0.02) -> Mesh:
    rng = _rng(seed)
    centers = rng.random((n_tris, 1, 3))
    offs = rng.uniform(-offset, offset, size=(n_tris, 3, 3))
    pos = (centers + offs).astype(F32).reshape(-1, 3)
    return Mesh(np.ascontiguousarray(pos), None)


def heightfield_params(seed: int) -> tuple[np.ndarray, np.ndarray]:
    rng = _rng(seed)
    theta = rng.uniform(0.0, 2.0 * math.pi, size=4)
    phi = rng.uniform(0.0, 2.0 * math.pi, size=4)
    return theta, phi


def heightfield_z(x: np.ndarray, y: np.ndarray, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    z = np.zeros(np.broadcast(x, y).shape, dtype=np.float64)
    for o, k in enumerate((2, 4, 8, 16)):
        z += (0.1 / k) * np.sin(2.0 * math.pi * k * (x * math.cos(theta[o]) + y * math.sin(theta[o])) + phi[o])
    return z


def heightfield(n: int = 1024, seed: int = 1, jitter_sigma: float = 0.0, jitter_seed: int | None = None) -> Mesh:
    """n x n vertex grid over [0,1]^2; vertex (i, j) has index j*n + i."""
    theta, phi = heightfield_params(seed)
    g = np.arange(n, dtype=np.float64) / (n - 1)
    x, y = np.meshgrid(g, g, indexing="xy")  # x varies along columns (i), y along rows (j)
    z = heightfield_z(x, y, theta, phi)
    if jitter_sigma > 0.0:
        jr = _rng(seed + 7919 if jitter_seed is None else jitter_seed)
        z = z + jr.normal(0.0, jitter_sigma, size=z.shape)
    pos = np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(F32)
    return Mesh(np.ascontiguousarray(pos), grid_indices(n))


def grid_indices(n: int) -> np.ndarray:
    j, i = np.meshgrid(np.arange(n - 1, dtype=np.uint32), np.arange(n - 1, dtype=np.uint32), indexing="ij")
    v00 = j * n + i
    v10 = v00 + 1
    v01 = v00 + n
    v11 = v01 + 1
    tris = np.stack([np.stack([v00, v10, v11], -1), np.stack([v00, v11, v01], -1)], axis=2)  # (n-1, n-1, 2, 3)
    return np.ascontiguousarray(tris.reshape(-1).astype(np.uint32))


def _normalize_f32(d: np.ndarray) -> np.ndarray:
    """normalize() with the reference's order: mag_sq = x*x + y*y + z*z, v * (1/sqrt(mag_sq))."""
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    mag_sq = (x * x + y * y) + z * z
    inv = F32(1.0) / np.sqrt(mag_sq)
    return np.stack([x * inv, y * inv, z * inv], axis=-1).astype(F32)


@dataclass
class PinholeCamera:
    """Pinhole camera as the f32 basis every ray generator (host or device) uses.

    direction(px, py) = normalize(forward + sx * right + sy * up) with
    sx = ((px + 0.5) / W * 2 - 1) * tan_half * aspect and
    sy = (1 - (py + 0.5) / H * 2) * tan_half, all in float32, left to right.
    """

    origin: np.ndarray
    forward: np.ndarray
    right: np.ndarray
    up: np.ndarray
    tan_half: np.float32
    aspect: np.float32
    width: int
    height: int

    @staticmethod
    def look_at(eye, target, vfov_deg: float, width: int, height: int, world_up=(0.0, 0.0, 1.0)) -> "PinholeCamera":
        eye64 = np.asarray(eye, np.float64)
        f = np.asarray(target, np.float64) - eye64
        f /= np.linalg.norm(f)
        r = np.cross(f, np.asarray(world_up, np.float64))
        if np.linalg.norm(r) < 1e-12:
            r = np.cross(f, np.array([0.0, 1.0, 0.0]))
        r /= np.linalg.norm(r)
        u = np.cross(r, f)
        return PinholeCamera(
            origin=eye64.astype(F32),
            forward=f.astype(F32),
            right=r.astype(F32),
            up=u.astype(F32),
            tan_half=F32(math.tan(math.radians(vfov_deg) / 2.0)),
            aspect=F32(width / height),
            width=width,
            height=height,
        )

    def as_floats(self) -> np.ndarray:
        """[origin, forward, right, up, tan_half, aspect] as 14 float32 values."""
        return np.concatenate(
            [self.origin, self.forward, self.right, self.up, np.array([self.tan_half, self.aspect], F32)]
        ).astype(F32)

    def directions(self) -> np.ndarray:
        W, H = self.width, self.height
        px = np.arange(W, dtype=F32)[None, :]
        py = np.arange(H, dtype=F32)[:, None]
        sx = ((px + F32(0.5)) / F32(W) * F32(2.0) - F32(1.0)) * self.tan_half * self.aspect
        sy = (F32(1.0) - (py + F32(0.5)) / F32(H) * F32(2.0)) * self.tan_half
        sx = np.broadcast_to(sx, (H, W))
        sy = np.broadcast_to(sy, (H, W))
        d = np.empty((H, W, 3), F32)
        for c in range(3):
            d[..., c] = (self.forward[c] + sx * self.right[c]) + sy * self.up[c]
        return _normalize_f32(d).reshape(-1, 3)


RAY_DTYPE = np.dtype([("org", F32, 3), ("tmin", F32), ("dir", F32, 3), ("tmax", F32)])  # 32 B


def make_rays(origins: np.ndarray, dirs: np.ndarray, tmin: float = 0.0, tmax: float = float("inf")) -> np.ndarray:
    n = dirs.shape[0]
    r = np.zeros(n, RAY_DTYPE)
    r["org"] = np.broadcast_to(np.asarray(origins, F32), (n, 3))
    r["dir"] = dirs
    r["tmin"] = F32(tmin)
    r["tmax"] = F32(tmax)
    return r


def pinhole_rays(camera: PinholeCamera, tmin: float = 0.0, tmax: float = float("inf")) -> np.ndarray:
    return make_rays(camera.origin, camera.directions(), tmin, tmax)


def soup_camera(width: int = 256, height: int = 256) -> PinholeCamera:
    """Plain closest-hit workload camera: eye (0.5,0.5,-1.5), looking +z, 60 deg vertical FOV."""
    return PinholeCamera(
        origin=np.array([0.5, 0.5, -1.5], F32),
        forward=np.array([0.0, 0.0, 1.0], F32),
        right=np.array([1.0, 0.0, 0.0], F32),
        up=np.array([0.0, 1.0, 0.0], F32),
        tan_half=F32(math.tan(math.radians(30.0))),
        aspect=F32(width / height),
        width=width,
        height=height,
    )


def heightfield_camera(width: int = 1920, height: int = 1080, vfov_deg: float = 20.0) -> PinholeCamera:
    """Wavefront workload camera: eye (0.5,-0.5,0.8) aimed at the grid centre (0.5,0.5,0).
    A 20 degree vertical field of view keeps the far edge of the grid (10.6 degrees
    above the view axis) and the near edge (19.3 degrees below) in frame, so almost
    every primary ray hits the field and spawns a shadow and a bounce ray."""
    return PinholeCamera.look_at((0.5, -0.5, 0.8), (0.5, 0.5, 0.0), vfov_deg, width, height)


def sphere_rays(n: int, box_min, box_max, seed: int, tmin: float = 0.0, tmax: float = float("inf")) -> np.ndarray:
    rng = _rng(seed)
    lo = np.asarray(box_min, np.float64)
    hi = np.asarray(box_max, np.float64)
    org = (lo + (hi - lo) * rng.random((n, 3))).astype(F32)
    z = rng.uniform(-1.0, 1.0, n)
    a = rng.uniform(0.0, 2.0 * math.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d = np.stack([s * np.cos(a), s * np.sin(a), z], -1).astype(F32)
    return make_rays(org, _normalize_f32(d), tmin, tmax)


def log_uniform_ints(n: int, lo: float, hi: float, seed: int) -> np.ndarray:
    rng = _rng(seed)
    return np.exp(rng.uniform(math.log(lo), math.log(hi), n)).astype(np.int64)


@dataclass
class BatchedScenes:
    """Many independent triangle soups with rays of uneven count per scene."""

    meshes: list
    rays: np.ndarray       # all scenes' rays, grouped by scene
    tlas_idx: np.ndarray   # scene index of every ray
    ray_offsets: np.ndarray  # rays of scene s are rays[ray_offsets[s]:ray_offsets[s+1]]


def batched_soups(n_scenes: int = 256, tri_range=(1_000, 200_000), ray_range=(4_096, 262_144), seed: int = 2,
                  offset: float = 0.02) -> BatchedScenes:
    """Batched workload: soups generated as triangle_soup with log-uniform
    triangle counts, rays per scene log-uniform, origins uniform in the scene's
    box [-offset, 1+offset]^3 and directions uniform on the sphere."""
    tris = log_uniform_ints(n_scenes, tri_range[0], tri_range[1], seed)
    nrays = log_uniform_ints(n_scenes, ray_range[0], ray_range[1], seed + 1)
    meshes, rays, idx = [], [], []
    for s in range(n_scenes):
        meshes.append(triangle_soup(int(tris[s]), seed=1000 + s, offset=offset))
        rays.append(sphere_rays(int(nrays[s]), (-offset,) * 3, (1 + offset,) * 3, seed=50_000 + s))
        idx.append(np.full(int(nrays[s]), s, np.uint32))
    offs = np.concatenate([[0], np.cumsum(nrays)]).astype(np.int64)
    return BatchedScenes(meshes, np.concatenate(rays), np.concatenate(idx), offs)
