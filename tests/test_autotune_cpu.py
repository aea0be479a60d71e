"""Host logic of the launch autotuner (timing uses CUDA events only on a GPU)."""

import json

from rendiation_gb300.autotune import Autotuner, grid


def test_grid_is_the_cartesian_product():
    g = grid(a=[1, 2], b=["x", "y", "z"])
    assert len(g) == 6
    assert {"a": 2, "b": "y"} in g


def test_cached_choice_is_reused(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text(json.dumps({"wf": {"best": {"block": 64}, "timings_ms": [[{"block": 64}, 1.0]]}}))
    t = Autotuner(str(path))
    r = t.tune("wf", grid(block=[32, 64]), run=lambda c: (_ for _ in ()).throw(AssertionError("no timing")))
    assert r.cached and r.best == {"block": 64}
