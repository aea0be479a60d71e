"""Launch-parameter autotuner.

The reference hard-codes its launch shapes (workgroup 128/256,
shader/task-graph/src/runtime/mod.rs:16,295; 512^2 launch strips,
shader/ray-tracing/src/backend/wavefront_compute/mod.rs:134). Here the knobs
that decide GB300 throughput are chosen per workload by timing every candidate
on the workload itself:

* node layout of the ordered traversal (2-wide or 4-wide nodes),
* block size (warps per block: occupancy against shared-memory stack size),
* ray-sort key of the batched executor (none, scene+octant, scene+octant+cell).

The traversal stack depth is not a knob: a stack walk without restarts needs
the tree depth, so it is derived from the built tree.

Each candidate is warmed up and then timed with CUDA events on the current
stream; the median decides. Choices are cached in a JSON file (keyed by a
workload signature) so that later runs reuse them without re-timing.
"""

from __future__ import annotations

import itertools
import json
import os
from dataclasses import dataclass, field


@dataclass
class TuneResult:
    best: dict
    timings_ms: list = field(default_factory=list)  # (candidate, median ms)
    cached: bool = False


def grid(**knobs) -> list[dict]:
    """Cartesian product of knob values as a list of candidate dicts."""
    names = list(knobs)
    return [dict(zip(names, vals)) for vals in itertools.product(*(knobs[n] for n in names))]


class Autotuner:
    def __init__(self, cache_path: str | None = None):
        self.cache_path = cache_path
        self.cache = {}
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as f:
                self.cache = json.load(f)

    def _save(self):
        if self.cache_path:
            os.makedirs(os.path.dirname(os.path.abspath(self.cache_path)), exist_ok=True)
            with open(self.cache_path, "w") as f:
                json.dump(self.cache, f, indent=1, sort_keys=True)

    def tune(self, key: str, candidates: list[dict], run, reps: int = 3, warmup: int = 1,
             use_cache: bool = True) -> TuneResult:
        """run(candidate) launches the workload once on the current CUDA stream."""
        import torch

        if use_cache and key in self.cache:
            return TuneResult(best=self.cache[key]["best"], timings_ms=self.cache[key]["timings_ms"], cached=True)
        stream = torch.cuda.current_stream()
        timings = []
        for cand in candidates:
            for _ in range(warmup):
                run(cand)
            samples = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                run(cand)
                e1.record(stream)
                e1.synchronize()
                samples.append(e0.elapsed_time(e1))
            samples.sort()
            timings.append((cand, samples[len(samples) // 2]))
        best = min(timings, key=lambda t: t[1])[0]
        self.cache[key] = {"best": best, "timings_ms": [[c, round(ms, 4)] for c, ms in timings]}
        self._save()
        return TuneResult(best=best, timings_ms=self.cache[key]["timings_ms"])
