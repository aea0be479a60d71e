"""GPU tests of the parallel-compute primitives (rdn_scan_u32, rdn_compact_u32,
rdn_radix_sort_u32) with the reference's own known-answer vectors
(shader/parallel-compute/src/prefix_scan.rs:122-172, stream_compaction.rs:100-125,
radix_sort.rs:143-154) and large random inputs against numpy."""

import ctypes as C

import numpy as np
import pytest
import torch

from rendiation_gb300 import native

pytestmark = pytest.mark.gpu


def scratch(kind, n):
    L = native.lib()
    size = C.c_size_t()
    assert getattr(L, f"rdn_{kind}_scratch_size")(n, C.byref(size)) == 0
    buf = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
    return buf, (buf.data_ptr() + 255) & ~255, size.value


def scan(x: np.ndarray, inclusive=True, segment=0) -> np.ndarray:
    L = native.lib()
    n = x.shape[0]
    d_in = torch.from_numpy(x.astype(np.int64).astype(np.uint32).view(np.int32)).cuda()
    d_out = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    keep, sp, sb = scratch("scan", n)
    assert L.rdn_scan_u32(d_in.data_ptr(), d_out.data_ptr(), n, int(inclusive), segment, sp, sb, None) == 0
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint32)[:n]


def test_scan_known_answers(cuda):
    ones = np.ones(70, np.uint32)
    # prefix_scan.rs:147-172: device-wide inclusive scan of 70 ones
    assert scan(ones).tolist() == list(range(1, 71))
    # prefix_scan.rs:122-145: workgroup-scoped (32) inclusive scan restarts every 32
    expect, s = [], 0
    for i in range(70):
        s = 1 if i % 32 == 0 else s + 1
        expect.append(s)
    assert scan(ones, segment=32).tolist() == expect


@pytest.mark.parametrize("n", [1, 2047, 2048, 2049, 100_000, 5_000_000])
def test_scan_random(n, cuda):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 1 << 20, n).astype(np.uint32)
    inc = np.cumsum(x.astype(np.uint64)).astype(np.uint32)
    assert np.array_equal(scan(x, True), inc)
    assert np.array_equal(scan(x, False), inc - x)
    seg = 1024
    xs = x.astype(np.uint64).reshape(-1)
    expect = np.concatenate([np.cumsum(xs[i:i + seg]) for i in range(0, n, seg)]).astype(np.uint32)
    assert np.array_equal(scan(x, True, seg), expect)


def compact(values, flags):
    L = native.lib()
    n = values.shape[0]
    dv = torch.from_numpy(values.astype(np.uint32).view(np.int32)).cuda()
    df = torch.from_numpy(flags.astype(np.uint32).view(np.int32)).cuda()
    out = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    keep, sp, sb = scratch("compact", n)
    assert L.rdn_compact_u32(dv.data_ptr(), df.data_ptr(), out.data_ptr(), cnt.data_ptr(), n, sp, sb, None) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32), int(cnt.item())


def test_compaction_known_answer(cuda):
    # stream_compaction.rs:100-125: [1,0,1,0,1,1,0] keeping the ones -> [1,1,1,1,0,0,0], size 4
    v = np.array([1, 0, 1, 0, 1, 1, 0], np.uint32)
    out, cnt = compact(v, (v == 1).astype(np.uint32))
    assert out.tolist() == [1, 1, 1, 1, 0, 0, 0]
    assert cnt == 4


def test_compaction_random(cuda):
    rng = np.random.default_rng(3)
    n = 3_000_001
    v = rng.integers(1, 1 << 31, n).astype(np.uint32)
    f = (rng.random(n) < 0.37).astype(np.uint32) * rng.integers(1, 5, n).astype(np.uint32)
    out, cnt = compact(v, f)
    keep = v[f != 0]
    assert cnt == keep.shape[0]
    assert np.array_equal(out[:cnt], keep)
    assert np.all(out[cnt:] == 0)


def sort(keys, vals=None, bits=32):
    L = native.lib()
    n = keys.shape[0]
    dk = torch.from_numpy(keys.astype(np.uint32).view(np.int32)).cuda()
    dv = None if vals is None else torch.from_numpy(vals.astype(np.uint32).view(np.int32)).cuda()
    keep, sp, sb = scratch("radix_sort", n)
    assert L.rdn_radix_sort_u32(dk.data_ptr(), None if dv is None else dv.data_ptr(), n, bits, sp, sb, None) == 0
    torch.cuda.synchronize()
    return dk.cpu().numpy().view(np.uint32), None if dv is None else dv.cpu().numpy().view(np.uint32)


def test_radix_sort_known_answer(cuda):
    # radix_sort.rs:143-154
    k, _ = sort(np.array([3, 1, 4, 6, 5, 2], np.uint32))
    assert k.tolist() == [1, 2, 3, 4, 5, 6]


@pytest.mark.parametrize("n,bits", [(1025, 32), (1_000_000, 32), (2_500_000, 12), (777, 3)])
def test_radix_sort_stable_pairs(n, bits, cuda):
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(0, 1 << bits, n).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = sort(keys, vals, bits)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order])
    assert np.array_equal(v, vals[order])  # stability: equal keys keep their input order
