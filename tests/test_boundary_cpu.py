"""CPU tests of the C-ABI boundary: exported symbols, host-side build parity
with the oracle (every flattened array byte for byte), handle and error
behaviour. No compute call touches a GPU."""

import ctypes as C
import os
import re

import numpy as np
import pytest

from helpers import ROOT, Scene, instanced_scene, orc, rt, scenes, single_mesh_scene
from rendiation_gb300 import native


def header_functions():
    txt = open(os.path.join(ROOT, "include", "rdn.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"typedef\s+rdn_status\s*\(\*[^;]*;", "", txt)  # function-pointer types
    return sorted(set(re.findall(r"\b(rdn_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = native.lib()
    declared = header_functions()
    assert declared, "no declarations parsed"
    assert sorted(native.EXPORTED_SYMBOLS) == declared
    for name in declared:
        assert hasattr(L, name), name
    assert L.rdn_api_version() == 1


def assert_same_arrays(sc: Scene):
    S = sc.build_oracle()
    P = sc.build_product(device=-1)
    for i, name in enumerate(rt.BUILT_ARRAYS):
        assert S.buffer(i) == P.built_array(name), name


def test_build_parity_soup():
    assert_same_arrays(single_mesh_scene(scenes.triangle_soup(10_000, seed=0)))


def test_build_parity_heightfield_bin2():
    assert_same_arrays(single_mesh_scene(scenes.heightfield(96, seed=3), bins=2))


def test_build_parity_degenerate_median_fallback():
    """Clustered centres force the BalanceTree median split (Rust select_nth_unstable)."""
    rng = np.random.default_rng(3)
    n = 4000
    c = np.where(rng.random((n, 1, 3)) < 0.97, 0.5, rng.random((n, 1, 3)))
    c = np.round(c * 8) / 8
    pos = (c + rng.uniform(-0.3, 0.3, (n, 3, 3))).astype(np.float32).reshape(-1, 3)
    sc = single_mesh_scene(scenes.Mesh(pos, None), bins=2)
    S = sc.build_oracle()
    assert S.build_stats()["median_fallbacks"] > 100
    assert_same_arrays(sc)


def test_build_parity_instances_and_deleted_slots():
    assert_same_arrays(instanced_scene(seed=5))


def test_per_geometry_root_box_quirk_is_mirrored():
    """A two-geometry BLAS followed by another BLAS: the reference indexes its
    per-geometry box list by BLAS handle (naive/mod.rs:239,272-275) and panics
    on the resulting None; oracle and product both report an error instead."""
    a = scenes.triangle_soup(50, seed=1)
    b = scenes.triangle_soup(50, seed=2)
    sc = Scene([[(a.positions, None, 1), (b.positions, None, 1)], [(b.positions, None, 1)], [(a.positions, None, 1)]],
               [[{"blas": 2}]], deleted_blas=[1])
    with pytest.raises(RuntimeError):
        sc.build_oracle()
    with pytest.raises(native.RdnError) as e:
        sc.build_product(device=-1)
    assert e.value.status == -2


def test_build_parity_empty_and_tiny_geometries():
    one = scenes.triangle_soup(1, seed=1)
    three = scenes.triangle_soup(3, seed=2)
    empty = np.zeros((0, 3), np.float32)
    sc = Scene([[(one.positions, None, 1)], [(three.positions, None, 0), (empty, None, 1)]],
               [[{"blas": 0}, {"blas": 1}], []], bind=[0, 1])
    assert_same_arrays(sc)


def test_host_only_context_rejects_trace():
    P = single_mesh_scene(scenes.triangle_soup(10, seed=1)).build_product(device=-1)
    d = native.TraceDesc(16, 16, 0, 0, 1, 0, 0, 0xFF, 0, 0, 0, 0)
    st = native.lib().rdn_trace(P._h, C.byref(d), None)
    assert st == -8  # RDN_ERR_UNSUPPORTED


def test_errors_are_status_codes():
    L = native.lib()
    P = rt.AccelerationStructureSystem(device=-1)
    with pytest.raises(native.RdnError) as e:
        P.delete_bottom_level_acceleration_structure(3)
    assert e.value.status == -2
    bad = scenes.Mesh(np.zeros((3, 3), np.float32), np.array([0, 1, 5], np.uint32))
    with pytest.raises(native.RdnError) as e:
        P.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(bad.positions, bad.indices)])
    assert e.value.status == -1
    b = P.create_bottom_level_acceleration_structure(
        [rt.BottomLevelAccelerationStructureBuildSource(scenes.triangle_soup(4, seed=0).positions)])
    P.delete_bottom_level_acceleration_structure(b)
    t = P.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(b)])
    P.bind_tlas([t])
    with pytest.raises(native.RdnError) as e:
        P.build()  # the instance points at a deleted BLAS (the reference panics on unwrap)
    assert e.value.status == -2
    size = C.c_size_t()
    assert L.rdn_get_built_array(P._h, 99, None, 0, C.byref(size)) in (-1, -7)
    h = C.c_void_p()
    assert L.rdn_create(C.byref(h), -5) == -1
    assert L.rdn_destroy(None) == -1


def test_handles_are_dense_and_deleted_slots_stay_empty():
    P = rt.AccelerationStructureSystem(device=-1)
    src = [rt.BottomLevelAccelerationStructureBuildSource(scenes.triangle_soup(4, seed=0).positions)]
    hs = [P.create_bottom_level_acceleration_structure(src) for _ in range(3)]
    assert hs == [0, 1, 2]
    P.delete_bottom_level_acceleration_structure(1)
    assert P.create_bottom_level_acceleration_structure(src) == 3
    with pytest.raises(native.RdnError):
        P.delete_bottom_level_acceleration_structure(1)


def test_device_build_needs_a_device():
    """A host-only context refuses the device build instead of building on the host."""
    sc = single_mesh_scene(scenes.triangle_soup(100, seed=1))
    with pytest.raises(native.RdnError) as ex:
        sc.build_product(device=-1, device_build=True)
    assert ex.value.status == -8  # RDN_ERR_UNSUPPORTED
