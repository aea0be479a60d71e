"""The committed golden fixtures (tests/golden/*.npz, written by
tests/golden/make_golden.py) against the oracle rebuilt on this machine, and
the product's host build against the fixtures' array digests.

The fixtures are oracle outputs (the Rust reference cannot be built here);
these tests pin the oracle across compilers and CPU architectures and pin the
product's flattened arrays to the same bytes without a GPU."""

import hashlib

import numpy as np
import pytest

import golden_cases as gc
from helpers import orc, rt


def same_bits(a, b):
    assert a.dtype == b.dtype
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))


def test_soup_oracle_reproduces_golden():
    g = gc.load("soup1k")
    S = gc.soup_scene(g).build_oracle()
    assert gc.digests_of_oracle(S) == g["digests"].tolist()
    rays = gc.rays_of(g)
    closest, _, cnt = S.trace(rays, counts=True)
    first, _ = S.trace(rays, ray_flags=rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH)
    same_bits(closest, g["closest"])
    same_bits(first, g["first"])
    assert np.array_equal(cnt, g["counts"])
    assert (g["closest"]["prim"] != orc.MISS).mean() > 0.25


@pytest.mark.parametrize("case", range(len(gc.FLAG_CASES)))
def test_instanced_oracle_reproduces_golden(case):
    g = gc.load("instanced")
    S = gc.instanced(g).build_oracle()
    assert gc.digests_of_oracle(S) == g["digests"].tolist()
    flags, mask = gc.FLAG_CASES[case]
    hits, _ = S.trace(gc.rays_of(g), tlas_idx=g["tlas_idx"], ray_flags=flags, cull_mask=mask)
    same_bits(hits, g[f"hits{case}"])


def test_wavefront_oracle_reproduces_golden():
    g = gc.load("wavefront")
    S = gc.wavefront_scene(g).build_oracle()
    pix, rays, _ = orc.wavefront_shadow_bounce(S, g["camera"], 48, 32, g["light"], int(g["sample_index"]))
    same_bits(pix, g["pixels"])
    assert rays == g["ray_counts"].tolist()


@pytest.mark.parametrize("name", ["soup1k", "instanced"])
def test_product_host_build_matches_golden_digests(name):
    g = gc.load(name)
    sc = gc.soup_scene(g) if name == "soup1k" else gc.instanced(g)
    P = sc.build_product(device=-1)
    got = [hashlib.sha256(P.built_array(a)).hexdigest() for a in rt.BUILT_ARRAYS]
    assert got == g["digests"].tolist()
