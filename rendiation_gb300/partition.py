"""Work partitioning across GPUs (one process per GPU).

The ray-query path shards without any exchange on its data path: rays are
independent, and so are the scenes of a batch. Each rank keeps a replica of
what it traces and works on its own share:

- a frame is split into contiguous row bands, one per rank
  (``row_bands``); rdn_wavefront_shadow_bounce traces a band with the whole
  frame's camera rays and samplers, so the bands' pixel records put together
  equal the frame's;
- a batch of scenes is split so that every rank gets about the same sum of
  triangles x rays (``balanced_scenes``, longest-processing-time greedy), the
  cost model of a traversal whose work grows with both;
- gradients of a differentiable batch are summed across ranks with one
  all-reduce after the backward pass (``sum_gradients``); scenes own disjoint
  vertices, so the sum is each rank's share in place.

The reference has no multi-GPU code; the per-ray scene key it would split on
is the TLAS index (``traverse_cpu.rs:63``).
"""

from __future__ import annotations

import numpy as np


def row_bands(height: int, world: int) -> list[tuple[int, int]]:
    """Contiguous bands [row0, row1) covering rows [0, height) once, in rank
    order, sizes differing by at most one row."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    base, extra = divmod(height, world)
    bands, r = [], 0
    for k in range(world):
        n = base + (1 if k < extra else 0)
        bands.append((r, r + n))
        r += n
    return bands


def balanced_scenes(costs, world: int) -> list[list[int]]:
    """Scene ids per rank: the heaviest remaining scene goes to the least
    loaded rank (ties to the lower rank), so the largest rank load is at most
    4/3 of the optimum plus one scene; deterministic for given costs. Each
    rank's list is in ascending scene order."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    c = np.asarray(costs, np.float64)
    order = sorted(range(c.size), key=lambda i: (-c[i], i))
    load = [0.0] * world
    owner = [[] for _ in range(world)]
    for i in order:
        k = min(range(world), key=lambda r: (load[r], r))
        owner[k].append(i)
        load[k] += float(c[i])
    return [sorted(o) for o in owner]


def scene_costs(triangles, rays) -> np.ndarray:
    """Per-scene cost: triangles x rays."""
    return np.asarray(triangles, np.float64) * np.asarray(rays, np.float64)


def batch_subset(batch, scene_ids):
    """The scenes `scene_ids` of a scenes.BatchedScenes with their rays,
    renumbered 0..k-1 in the given order (the rank's own batch)."""
    from .scenes import BatchedScenes

    ids = [int(i) for i in scene_ids]
    meshes = [batch.meshes[i] for i in ids]
    rays = [batch.rays[batch.ray_offsets[i]:batch.ray_offsets[i + 1]] for i in ids]
    counts = [r.shape[0] for r in rays]
    idx = np.concatenate([np.full(c, k, np.uint32) for k, c in enumerate(counts)]) if ids else np.zeros(0, np.uint32)
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return BatchedScenes(meshes, np.concatenate(rays) if ids else batch.rays[:0], idx, offs)


def sum_gradients(grad, group=None):
    """Sums a gradient tensor across the ranks of torch.distributed's group in
    place (one all-reduce); a no-op without an initialised process group."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
    return grad
