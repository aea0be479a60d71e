"""Multi-GPU partitioning (rendiation_gb300.partition) on CPU, with
world_size-2 gloo ranks standing in for two GPUs:

- row bands of a frame cover every row exactly once, and the oracle's
  pipeline over each rank's band gives, put together, the whole frame's pixel
  records (the product's band launches are checked against whole frames on
  the GPU in tests/test_wavefront_gpu.py);
- the balanced scene split gives every scene to exactly one rank, within the
  greedy bound of the optimum;
- vertex gradients computed per rank on its own scenes and summed with one
  all-reduce equal the gradients of one rank doing every scene."""

import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from rendiation_gb300 import partition  # noqa: E402

LIGHT = (0.2, 0.2, 2.0)


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("height,world", [(1080, 1), (1080, 2), (1080, 8), (7, 3), (3, 8), (0, 2)])
def test_row_bands_cover_every_row_once(height, world):
    bands = partition.row_bands(height, world)
    assert len(bands) == world
    rows = np.concatenate([np.arange(a, b) for a, b in bands]) if height else np.zeros(0)
    assert np.array_equal(rows, np.arange(height))
    sizes = [b - a for a, b in bands]
    assert max(sizes) - min(sizes) <= 1


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_balanced_scenes(world):
    rng = np.random.default_rng(world)
    tris = np.exp(rng.uniform(np.log(1e3), np.log(2e5), 256)).astype(np.int64)
    rays = np.exp(rng.uniform(np.log(4e3), np.log(2.6e5), 256)).astype(np.int64)
    c = partition.scene_costs(tris, rays)
    owner = partition.balanced_scenes(c, world)
    flat = sorted(i for o in owner for i in o)
    assert flat == list(range(256))
    loads = [c[o].sum() for o in owner]
    assert max(loads) <= c.sum() / world + c.max()
    assert partition.balanced_scenes(c, world) == owner  # deterministic


def scenes_for_test():
    from helpers import scenes

    return [scenes.heightfield(g, seed=40 + k) for k, g in enumerate([8, 14, 11, 20, 9])]


def gradients(meshes, which):
    """FP64 gradient of sum over rays of (interpolated attribute - 0.3)^2 with
    respect to every vertex's position and attribute, frozen visibility, over
    the scenes in `which`; the oracle (the CPU restatement of the reference's
    traversal) finds each ray's triangle. Scenes' vertices are concatenated."""
    from helpers import scenes, single_mesh_scene

    offs = np.cumsum([0] + [m.positions.shape[0] for m in meshes])
    g = np.zeros((offs[-1], 4))
    for k in which:
        m = meshes[k]
        S = single_mesh_scene(m).build_oracle()
        cam = scenes.PinholeCamera.look_at((0.5, -0.4, 0.8), (0.5, 0.5, 0.0), 30.0, 24, 16)
        rays = scenes.pinhole_rays(cam)
        hits, _ = S.trace(rays, threads=1)
        hit = hits["prim"] != 0xFFFFFFFF
        tv = m.indices.reshape(-1, 3)[hits["prim"][hit]]
        pos = m.positions.astype(np.float64)
        attr = np.linspace(0.0, 1.0, m.positions.shape[0])
        o = rays["org"][hit].astype(np.float64)
        d = rays["dir"][hit].astype(np.float64)
        v = pos[tv]
        M = np.stack([-d, v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]], axis=2)
        x = np.linalg.solve(M, (o - v[:, 0])[..., None])[..., 0]
        u, w = x[:, 1], x[:, 2]
        val = (1 - u - w) * attr[tv[:, 0]] + u * attr[tv[:, 1]] + w * attr[tv[:, 2]]
        r = 2 * (val - 0.3)
        G = np.stack([np.zeros_like(r), r * (attr[tv[:, 1]] - attr[tv[:, 0]]), r * (attr[tv[:, 2]] - attr[tv[:, 0]])], 1)
        lam = np.linalg.solve(np.transpose(M, (0, 2, 1)), G[..., None])[..., 0]
        for c, wc in enumerate([1 - u - w, u, w]):
            np.add.at(g[:, :3], offs[k] + tv[:, c], -wc[:, None] * lam)
            np.add.at(g[:, 3], offs[k] + tv[:, c], r * wc)
    return g


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        from helpers import orc, scenes, single_mesh_scene

        # (1) a frame split in row bands: each rank traces its band
        mesh = scenes.heightfield(48, seed=3)
        S = single_mesh_scene(mesh).build_oracle()
        cam = scenes.heightfield_camera(64, 37)
        r0, r1 = partition.row_bands(cam.height, ws)[rank]
        band, _, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), cam.width, cam.height, LIGHT, 5, row0=r0,
                                                 row1=r1, threads=1)
        parts = [None] * ws
        dist.all_gather_object(parts, (r0, r1, band.tobytes()))
        # (2) scenes split by triangles x rays, gradients summed with one all-reduce
        meshes = scenes_for_test()
        costs = partition.scene_costs([m.triangle_count for m in meshes], [24 * 16] * len(meshes))
        mine = partition.balanced_scenes(costs, ws)[rank]
        g = torch.from_numpy(gradients(meshes, mine))
        partition.sum_gradients(g)
        owners = [None] * ws
        dist.all_gather_object(owners, mine)
        q.put((rank, parts, g.numpy(), owners))
    finally:
        dist.destroy_process_group()


def test_two_ranks_partition_frame_and_scenes():
    from helpers import orc, scenes, single_mesh_scene

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # the bands tile the frame and give its records
    mesh = scenes.heightfield(48, seed=3)
    S = single_mesh_scene(mesh).build_oracle()
    cam = scenes.heightfield_camera(64, 37)
    full, _, _ = orc.wavefront_shadow_bounce(S, cam.as_floats(), cam.width, cam.height, LIGHT, 5, threads=1)
    for rank, parts, _, _ in res:
        rows = [r for a, b, _ in parts for r in range(a, b)]
        assert rows == list(range(cam.height))
        stacked = b"".join(p[2] for p in parts)
        assert stacked == full.tobytes()
    # every scene on exactly one rank; the reduced gradients equal one rank's
    owners = res[0][3]
    assert sorted(i for o in owners for i in o) == list(range(5))
    assert all(len(o) > 0 for o in owners)
    single = gradients(scenes_for_test(), range(5))
    for _, _, g, _ in res:
        assert np.array_equal(g, single)
