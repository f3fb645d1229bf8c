"""Builds libgb_gmg.so (the sm_103a CUDA library behind include/gb_gmg.h) in-tree.

    python -m aspect_gb300.build [--force]

Translation units are compiled in parallel with nvcc for sm_103a only and
linked into aspect_gb300/libgb_gmg.so; objects go to aspect_gb300/_build/.
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
LIB = os.path.join(HERE, "libgb_gmg.so")
SOURCES = ["kernels_f32.cu", "kernels_f64.cu", "adjoint.cu", "vec.cu", "level_setup.cu", "gb_gmg.cu", "noalloc.cu", "mass_bottom.cu", "ablock_fused.cu", "newton.cu", "coefficients.cu", "free_surface.cu", "ho_kernels.cu", "a_bottom.cu", "lattice_transfer.cu"]
# measured FP64/FP32 FMA peaks for the benchmark's rooflines (not part of the solver)
PROBE_LIB = os.path.join(HERE, "libgb_probe.so")
PROBE_SOURCES = ["peak_probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "gb_gmg.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    if (not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime() and os.path.exists(PROBE_LIB)
            and os.path.getmtime(PROBE_LIB) >= _deps_mtime()):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nv, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    all_sources = SOURCES + PROBE_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(len(all_sources), os.cpu_count() or 4)) as ex:
        objs = dict(zip(all_sources, ex.map(compile_one, all_sources)))
    for lib, srcs, libs in ((LIB, SOURCES, ["-lcudart", "-lcusolver", "-lcublas"]),
                            (PROBE_LIB, PROBE_SOURCES, ["-lcudart"])):
        tmp = lib + ".tmp"
        cmd = [nv, *ARCH, "-shared", "-o", tmp, *[objs[x] for x in srcs], *libs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
