"""Writes the golden fixtures of tests/golden/ from the oracle.

The reference is Rust and cannot be built in this environment, so its own
outputs cannot be recorded; these fixtures are the oracle's outputs on small,
fully stored inputs (raw float32/uint32 arrays, no generator needed to read
them). They pin the oracle across machines (x86_64 here, aarch64 on the GPU
host) and give the GPU parity tests a fixed answer that does not depend on
building the oracle at test time.

Cases:
  soup1k    1000-triangle soup, 64x64 pinhole rays: closest hits and first hits
            (reference order) with per-ray node-visit / triangle-test counts,
            and SHA-256 digests of every flattened array the build produces.
  instanced heightfield + two-geometry BLAS, a deleted BLAS slot, two TLAS with
            rotated / scaled / mirrored instances, masks, custom indices,
            culling and non-opaque flags; 4096 rays with origins in a box around the
            scene, both TLAS, five ray-flag / cull-mask combinations.
  wavefront 32x32 heightfield, 48x32 frame of the primary + shadow + bounce
            pipeline (pixel records).
  naive_fixture
            the reference's own BVH test scene (naive/test.rs:9-225: sphere, torus
            and cube BLAS, five TLAS) with its 256x256 back-face-culled camera:
            the generated vertex arrays and instance transforms, per TLAS the
            primitive-id image of test.rs:266-270 and the full hit records of
            every fourth pixel in both directions, and the build digests.

Run:  python tests/golden/make_golden.py [case ...]   (all cases when none is named)
"""

from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
sys.path.insert(0, TESTS)

from helpers import instanced_scene, orc, rt, scenes, single_mesh_scene  # noqa: E402
import naive_fixture as nf  # noqa: E402

LIGHT = np.array([0.2, 0.2, 2.0], np.float32)
FLAG_CASES = [
    (0, 0xFF),
    (rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH, 0xFF),
    (rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES, 0x03),
    (rt.RAY_FLAG_FORCE_NON_OPAQUE | rt.RAY_FLAG_CULL_NON_OPAQUE, 0xFF),
    (rt.RAY_FLAG_CULL_FRONT_FACING_TRIANGLES | rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH, 0x02),
]


def digests(S: orc.OracleSystem) -> np.ndarray:
    return np.array([hashlib.sha256(S.buffer(w)).hexdigest() for w in range(11)])


def soup_case():
    mesh = scenes.triangle_soup(1000, seed=11, offset=0.15)
    cam = scenes.soup_camera(64, 64)
    rays = scenes.pinhole_rays(cam)
    S = single_mesh_scene(mesh).build_oracle()
    closest, _, cnt = S.trace(rays, counts=True)
    first, _ = S.trace(rays, ray_flags=rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH)
    return dict(positions=mesh.positions, rays=rays.view(np.float32).reshape(-1, 8), closest=closest, first=first,
                counts=cnt, digests=digests(S))


def instanced_case():
    sc = instanced_scene(seed=0)
    S = sc.build_oracle()
    rays = scenes.sphere_rays(4096, (-0.5, -0.5, -0.5), (1.5, 1.5, 1.5), seed=5)
    tidx = (np.arange(rays.shape[0]) % 2).astype(np.uint32)
    out = {"rays": rays.view(np.float32).reshape(-1, 8), "tlas_idx": tidx, "digests": digests(S)}
    for k, (flags, mask) in enumerate(FLAG_CASES):
        out[f"hits{k}"], _ = S.trace(rays, tlas_idx=tidx, ray_flags=flags, cull_mask=mask)
    return out


def wavefront_case():
    mesh = scenes.heightfield(32, seed=3)
    cam = scenes.heightfield_camera(48, 32)
    S = single_mesh_scene(mesh).build_oracle()
    pix, nrays, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), 48, 32, LIGHT, sample_index=4)
    return dict(positions=mesh.positions, indices=mesh.indices, camera=cam.as_floats(), light=LIGHT,
                sample_index=np.uint32(4), pixels=pix, ray_counts=np.array(nrays, np.uint64))


def naive_fixture_case():
    ms = nf.meshes()
    S = nf.make_scene(ms).build_oracle()
    rays = nf.camera_rays(*nf.CPU_TEST_RANGE)
    out = {"digests": digests(S), "transforms": nf.all_transforms()}
    for name, m in zip(("sphere", "torus", "cube"), ms):
        out[f"{name}_positions"], out[f"{name}_indices"] = m.positions, m.indices
    for k in range(5):
        h, _ = S.trace(rays, tlas_uniform=k, ray_flags=rt.RAY_FLAG_CULL_BACK_FACING_TRIANGLES)
        out[f"image{k}"] = nf.id_image(h["prim"], orc.MISS)
        out[f"hits{k}"] = h.reshape(nf.H, nf.W)[::4, ::4].reshape(-1)
    return out


CASES = {"soup1k": soup_case, "instanced": instanced_case, "wavefront": wavefront_case,
         "naive_fixture": naive_fixture_case}


def main():
    names = sys.argv[1:] or list(CASES)
    for name, fn in ((n, CASES[n]) for n in names):
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **fn())
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
