"""Shared test helpers: one scene description, built into both the product
(librdn through its C ABI) and the oracle (the CPU restatement of the
reference), plus result comparison with tie classification."""

from __future__ import annotations

import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import orc  # noqa: E402
from rendiation_gb300 import raytracing as rt  # noqa: E402
from rendiation_gb300 import scenes  # noqa: E402


def mat4_cols(rot=np.eye(3), scale=(1.0, 1.0, 1.0), translate=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Mat4 in the reference's element order: columns a, b, c, d; translation in d."""
    m = np.eye(4)
    m[:3, :3] = np.asarray(rot) @ np.diag(scale)
    m[:3, 3] = translate
    return m.T.reshape(-1).astype(np.float32)  # column-major flatten


def rot_z(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])


def rot_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1.0, 0, 0], [0, c, -s], [0, s, c]])


class Scene:
    """blas: list of BLAS, each a list of (positions, indices|None, flags);
    tlas: list of TLAS, each a list of instance dicts (blas, transform, custom, mask, sbt, flags);
    bind: bound TLAS handles; deleted_blas / deleted_tlas: handles deleted after creation."""

    def __init__(self, blas, tlas, bind=None, deleted_blas=(), deleted_tlas=(), blas_bin_size=4, tlas_bin_size=10):
        self.blas = blas
        self.tlas = tlas
        self.bind = list(range(len(tlas))) if bind is None else list(bind)
        self.deleted_blas = list(deleted_blas)
        self.deleted_tlas = list(deleted_tlas)
        self.blas_bin_size = blas_bin_size
        self.tlas_bin_size = tlas_bin_size

    def build_oracle(self, blas_max_depth=50) -> orc.OracleSystem:
        S = orc.OracleSystem()
        for geoms in self.blas:
            S.create_blas(geoms)
        for inst in self.tlas:
            S.create_tlas(inst)
        for h in self.deleted_blas:
            S.delete_blas(h)
        for h in self.deleted_tlas:
            S.delete_tlas(h)
        S.bind_tlas(self.bind)
        S.build(blas_bin_size=self.blas_bin_size, tlas_bin_size=self.tlas_bin_size, blas_max_depth=blas_max_depth)
        return S

    def build_product(self, device=0, device_build=False, blas_max_depth=0) -> rt.AccelerationStructureSystem:
        P = rt.AccelerationStructureSystem(device=device)
        for geoms in self.blas:
            P.create_bottom_level_acceleration_structure(
                [rt.BottomLevelAccelerationStructureBuildSource(p, i, f) for p, i, f in geoms])
        for inst in self.tlas:
            P.create_top_level_acceleration_structure([
                rt.TopLevelAccelerationStructureSourceInstance(
                    s["blas"], s.get("transform", np.eye(4, dtype=np.float32).reshape(-1)), s.get("custom", 0),
                    s.get("mask", 0xFF), s.get("sbt", 0), s.get("flags", 0)) for s in inst])
        for h in self.deleted_blas:
            P.delete_bottom_level_acceleration_structure(h)
        for h in self.deleted_tlas:
            P.delete_top_level_acceleration_structure(h)
        P.bind_tlas(self.bind)
        P.build(blas_bin_size=self.blas_bin_size, tlas_bin_size=self.tlas_bin_size, blas_max_depth=blas_max_depth,
                device_build=device_build)
        return P


def single_mesh_scene(mesh: scenes.Mesh, flags=1, bins=4) -> Scene:
    return Scene([[(mesh.positions, mesh.indices, flags)]], [[{"blas": 0}]], blas_bin_size=bins)


def instanced_scene(seed=0) -> Scene:
    """Three BLAS slots: a heightfield, a deleted slot, and a BLAS with two
    geometries (opaque + non-opaque); two TLAS with rotated / scaled / mirrored
    instances, masks and custom indices. The two-geometry BLAS is last: the
    reference keeps one root box per geometry, not per BLAS (naive/mod.rs:239),
    so its instance bounds use the first geometry's box, and a BLAS placed after
    it would look up a shifted box."""
    a = scenes.triangle_soup(600, seed=seed + 1, offset=0.05)
    b = scenes.heightfield(24, seed=seed + 2)
    c = scenes.triangle_soup(300, seed=seed + 3, offset=0.08)
    blas = [
        [(b.positions, b.indices, 1)],                      # 0: heightfield
        [(c.positions, None, 1)],                           # 1: deleted below
        [(a.positions, None, 1), (c.positions, None, 0)],   # 2: two geometries, second non-opaque
    ]
    tlas = [
        [
            {"blas": 2, "custom": 7, "mask": 0x01},
            {"blas": 0, "transform": mat4_cols(rot_z(0.7), (1.5, 1.5, 0.5), (0.2, -0.3, 0.1)), "custom": 9,
             "mask": 0x03},
            {"blas": 0, "transform": mat4_cols(rot_x(0.3), (-1.0, 1.0, 1.0), (0.0, 0.8, 0.4)), "custom": 11,
             "mask": 0x02, "flags": rt.GEOMETRY_INSTANCE_TRIANGLE_FACING_CULL_DISABLE},
        ],
        [
            {"blas": 0, "transform": mat4_cols(np.eye(3), (2.0, 2.0, 2.0), (-0.5, -0.5, -0.5)), "custom": 3},
            {"blas": 2, "transform": mat4_cols(rot_z(-1.1), (0.8, 1.2, 1.0), (0.5, 0.5, 0.5)), "custom": 4,
             "flags": rt.GEOMETRY_INSTANCE_FORCE_NO_OPAQUE},
        ],
    ]
    return Scene(blas, tlas, bind=[1, 0], deleted_blas=[1])


def classify(got, expect, oracle_sys=None, rays=None):
    """Compare product hits with oracle hits. Returns dict with counts of
    identical results, exact-distance ties (same t, different primitive) and
    other mismatches."""
    g_hit = got["prim"] != orc.MISS
    e_hit = expect["prim"] != orc.MISS
    same_prim = got["prim"] == expect["prim"]
    same_t = got["t"] == expect["t"]
    identical = same_prim & ((~e_hit) | (same_t & (got["u"] == expect["u"]) & (got["v"] == expect["v"])))
    tie = (~identical) & g_hit & e_hit & same_t
    other = ~(identical | tie)
    return {"n": int(got.shape[0]), "identical": int(identical.sum()), "ties": int(tie.sum()),
            "other": int(other.sum()), "other_idx": np.nonzero(other)[0][:20].tolist(),
            "hit_mismatch": int((g_hit != e_hit).sum())}


def tilted_grid(g: int = 33) -> scenes.Mesh:
    """A g x g vertex grid on the tilted plane z = 0.3x + 0.2y over [0,1]^2, two
    triangles per cell, consistently wound: every interior edge is shared by
    two triangles that continue the same surface."""
    xs = np.linspace(0.0, 1.0, g, dtype=np.float32)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    Z = (np.float32(0.3) * X + np.float32(0.2) * Y).astype(np.float32)
    pos = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    q = []
    for j in range(g - 1):
        for i in range(g - 1):
            a = j * g + i
            q += [a, a + 1, a + g + 1, a, a + g + 1, a + g]
    return scenes.Mesh(pos, np.array(q, np.uint32))


def edge_rays(mesh: scenes.Mesh, n: int, seed: int, margin: float = 1e-3, vertex_share: float = 0.1) -> np.ndarray:
    """Rays aimed (in FP64) at points on triangle edges of `mesh` (a share of
    them exactly at vertices), from the front side of a surface facing +z,
    keeping only points at least `margin` inside [0,1]^2 (away from the mesh's
    outer boundary)."""
    rng = np.random.default_rng(seed)
    pos = mesh.positions.reshape(-1, 3)
    t3 = mesh.indices.reshape(-1, 3)
    tri = rng.integers(0, t3.shape[0], n)
    k = rng.integers(0, 3, n)
    a = pos[t3[tri, k]].astype(np.float64)
    b = pos[t3[tri, (k + 1) % 3]].astype(np.float64)
    s = rng.random(n) * 0.98 + 0.01
    s[: int(n * vertex_share)] = 0.0
    p = a + (b - a) * s[:, None]
    inner = (p[:, 0] > margin) & (p[:, 0] < 1 - margin) & (p[:, 1] > margin) & (p[:, 1] < 1 - margin)
    p = p[inner]
    d = rng.normal(size=(p.shape[0], 3))
    d[:, 2] = -np.abs(d[:, 2]) - 0.5
    d /= np.linalg.norm(d, axis=1)[:, None]
    return scenes.make_rays((p - 1.5 * d).astype(np.float32), d.astype(np.float32))
