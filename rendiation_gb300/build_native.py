"""Builds librdn.so in-tree with nvcc for sm_103a.

Host C++ is compiled with -ffp-contract=off (the precomputed f32 values must
equal the reference's un-fused arithmetic); the traversal kernels with
-fmad=false for the same reason. Translation units compile in parallel.
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librdn.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = "-O2,-fPIC,-ffp-contract=off,-fno-fast-math,-Wall,-Wno-unused-function"

# per-unit extra flags
UNITS = {
    "as_build.cpp": [],
    "rdn_api.cpp": [],
    "trace.cu": ["-fmad=false"],
    "wavefront.cu": ["-fmad=false"],
    "wavefront_static.cu": [],
    "paths.cu": ["-fmad=false"],
    "adjoint.cu": ["-fmad=false"],
    "parallel.cu": [],
    "device_build.cu": ["-fmad=false"],
    "task_graph.cu": ["-fmad=false"],
    "ao.cu": ["-fmad=false"],
    "pt.cu": ["-fmad=false"],
}


def _cmd(src: str, extra: list[str]) -> list[str]:
    out = os.path.join(OBJ, src + ".o")
    base = [NVCC, "-std=c++17", "-O3", "-Xcompiler", HOST_FLAGS, "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", out]
    if src.endswith(".cu"):
        base += ARCH + ["-lineinfo", "-Xptxas", "-O3"]
    else:
        base += ["-x", "c++"]
    return base + extra


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    cmds = []
    for src, extra in UNITS.items():
        e = list(extra)
        if ptxas_info and src.endswith(".cu"):
            e += ["-Xptxas", "-v"]
        cmds.append(_cmd(src, e))

    def run(c):
        if verbose:
            print(" ".join(c), flush=True)
        r = subprocess.run(c, capture_output=True, text=True)
        return c, r

    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        results = list(ex.map(run, cmds))
    for c, r in results:
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(c)}\n{r.stdout}\n{r.stderr}")
        if (verbose or ptxas_info) and r.stderr:
            print(r.stderr, file=sys.stderr)
    objs = [os.path.join(OBJ, s + ".o") for s in UNITS]
    link = [NVCC, "-shared", "-o", LIB] + objs + ARCH + ["-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
