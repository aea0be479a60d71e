"""The Python mirror of the C ABI (rendiation_gb300/native.py) against
include/rdn.h: every mirrored struct has the header's size and, field by
field, the header's offsets (a small C program compiled with the host
compiler prints them)."""

import ctypes as C
import os
import subprocess

import pytest

from helpers import ROOT
from rendiation_gb300 import native

PAIRS = [
    ("rdn_geometry", native.Geometry), ("rdn_instance", native.Instance), ("rdn_build_opts", native.BuildOpts),
    ("rdn_build_stats", native.BuildStats), ("rdn_trace_desc", native.TraceDesc), ("rdn_counters", native.Counters),
    ("rdn_camera", native.Camera), ("rdn_wavefront_desc", native.WavefrontDesc), ("rdn_path_desc", native.PathDesc),
    ("rdn_attr_loss_desc", native.AttrLossDesc), ("rdn_attr_path_desc", native.AttrPathDesc),
    ("rdn_hit_diff_desc", native.HitDiffDesc),
    ("rdn_task_group_desc", native.TaskGroupDesc), ("rdn_ao_desc", native.AoDesc), ("rdn_pt_desc", native.PtDesc),
]


@pytest.fixture(scope="module")
def header_layout(tmp_path_factory):
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "rdn.h"', "int main(void) {"]
    for cname, py in PAIRS:
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    layout = {}
    for line in out:
        if line:
            s, f, v = line.split()
            layout[(s, f)] = int(v)
    return layout


def test_path_tracing_records_match_header(header_layout, tmp_path):
    """rdn_pt_material / rdn_pt_directional_light against the numpy record types."""
    from rendiation_gb300 import path_tracing as pt

    src = tmp_path / "pt.c"
    names = {"rdn_pt_material": pt.MATERIAL_DTYPE, "rdn_pt_directional_light": pt.DIRECTIONAL_LIGHT_DTYPE}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "rdn.h"', "int main(void) {"]
    for cname, dt in names.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname in dt.names:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    src.write_text("\n".join(lines + ["  return 0;", "}"]) + "\n")
    exe = tmp_path / "pt"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    got = {(out[i], out[i + 1]): int(out[i + 2]) for i in range(0, len(out), 3)}
    for cname, dt in names.items():
        assert got[(cname, "sizeof")] == dt.itemsize
        for fname in dt.names:
            assert got[(cname, fname)] == dt.fields[fname][1], (cname, fname)


@pytest.mark.parametrize("cname,py", PAIRS, ids=[p[0] for p in PAIRS])
def test_struct_layout_matches_header(header_layout, cname, py):
    assert C.sizeof(py) == header_layout[(cname, "sizeof")], cname
    for fname, _ in py._fields_:
        assert getattr(py, fname).offset == header_layout[(cname, fname)], (cname, fname)
