"""The product's iterative restatement of Rust's select_nth_unstable_by (the
BVH median fallback; one copy serves the host build and the device build)
against the oracle's recursive restatement: identical permutations on tied,
sorted, reversed, organ-pipe, NaN-holding and random keys, through the normal
entry and through the median-of-medians worst-case path."""

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("select") / "libselect.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", out,
                    os.path.join(HERE, "select_harness.cpp")], check=True)
    lib = C.CDLL(out)
    lib.compare_select.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int]
    return lib


def key_sets(n, rng):
    yield rng.random(n).astype(np.float32)
    yield rng.integers(0, 4, n).astype(np.float32)            # heavy ties
    yield np.full(n, 0.5, np.float32)                          # all equal
    yield np.arange(n, dtype=np.float32)                       # sorted
    yield np.arange(n, 0, -1).astype(np.float32)               # reversed
    yield np.concatenate([np.arange(n // 2), np.arange(n - n // 2, 0, -1)]).astype(np.float32)  # organ pipe
    k = rng.random(n).astype(np.float32)
    k[rng.random(n) < 0.05] = np.nan
    yield k


@pytest.mark.parametrize("n", [2, 3, 17, 64, 65, 200, 1025, 5000, 140_000])
def test_select_matches_oracle(harness, n):
    rng = np.random.default_rng(n)
    for ks, keys in enumerate(key_sets(n, rng)):
        keys = np.ascontiguousarray(keys)
        for index in sorted({0, 1, n // 2, n - 1, int(rng.integers(0, n))}):
            for worst in (0, 1):
                if worst and ks == 2 and n > 5000:
                    # median-of-medians on all-equal keys shrinks the slice by one
                    # per partition (quadratic, in the library too); select itself
                    # never reaches it there (the equal-ancestor step ends first)
                    continue
                assert harness.compare_select(keys.ctypes.data, n, index, worst) == 1, (n, index, worst)
