"""Loads the golden fixtures of tests/golden/ (written by make_golden.py) and
rebuilds their scenes, for the oracle and for the product."""

from __future__ import annotations

import hashlib
import os

import numpy as np

from helpers import instanced_scene, orc, rt, scenes, single_mesh_scene

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FLAG_CASES = [
    (0, 0xFF),
    (rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH, 0xFF),
    (rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES, 0x03),
    (rt.RAY_FLAG_FORCE_NON_OPAQUE | rt.RAY_FLAG_CULL_NON_OPAQUE, 0xFF),
    (rt.RAY_FLAG_CULL_FRONT_FACING_TRIANGLES | rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH, 0x02),
]


def load(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as d:
        return {k: d[k] for k in d.files}


def rays_of(g: dict, key: str = "rays") -> np.ndarray:
    return np.ascontiguousarray(g[key]).view(scenes.RAY_DTYPE).reshape(-1)


def soup_scene(g: dict):
    p = np.ascontiguousarray(g["positions"], np.float32)
    return single_mesh_scene(scenes.Mesh(p, None))


def wavefront_scene(g: dict):
    return single_mesh_scene(scenes.Mesh(np.ascontiguousarray(g["positions"], np.float32),
                                         np.ascontiguousarray(g["indices"], np.uint32)))


def instanced(g: dict):
    return instanced_scene(seed=0)


def camera_of(g: dict, width: int, height: int):
    f = g["camera"].astype(np.float32)
    return scenes.PinholeCamera(origin=f[0:3], forward=f[3:6], right=f[6:9], up=f[9:12], tan_half=f[12],
                                aspect=f[13], width=width, height=height)


def digests_of_oracle(S: orc.OracleSystem) -> list[str]:
    return [hashlib.sha256(S.buffer(w)).hexdigest() for w in range(11)]
