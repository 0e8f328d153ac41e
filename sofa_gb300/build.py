"""Builds libsofa_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel; the FP64 reference-rounding
variant gets -fmad=false. Outputs: sofa_gb300/libsofa_gb300.so (objects in
sofa_gb300/_build/). Run: python -m sofa_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsofa_gb300.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off for the host compiler: host-side factor arithmetic (the
# implicit-Euler factors, the components' Rayleigh terms) rounds each a*b+c
# twice, as the reference does on a target without fused multiply-add; the
# Arm hosts' gcc would otherwise fuse it. Device code is governed by -fmad.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

# translation unit -> extra flags
UNITS = {
    "tfem_fp64_exact.cu": ["-fmad=false"],
    "tfem_fp64_fast.cu": ["-fmad=true"],
    "tfem_mixed.cu": ["-fmad=true"],
    "capi.cu": [],
    "mesh_layout.cu": [],
    "noalloc.cu": [],
    "von_mises.cu": ["-fmad=false"],
    "batch.cu": [],
    "server.cu": [],
    "scene_graph.cpp": [],
    "scene_components.cpp": [],
    "scene_xml.cpp": [],
    "plugin.cpp": [],
}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def _sources_mtime():
    latest = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            latest = max(latest, os.path.getmtime(os.path.join(d, f)))
    return max(latest, os.path.getmtime(__file__))


def up_to_date():
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime()


def _compile(unit, flags, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o").replace(".cpp", ".o"))
    cmd = [nvcc()] + ARCH + COMMON + flags + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, u, f, verbose) for u, f in UNITS.items()]
        objs = [f.result() for f in futs]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
