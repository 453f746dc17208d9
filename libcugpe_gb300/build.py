"""Builds libgpe_gb300.so in-tree for sm_103a (GB300).

The fused pass kernel is instantiated in one generated translation unit per
(precision, pencil length), compiled in parallel, then linked with the engine
and the drop-in API into ``libcugpe_gb300/_lib/libgpe_gb300.so``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libgpe_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
LENGTHS = [8, 16, 32, 64, 128, 256, 512]
PRECISIONS = {"f64": "double", "f32": "float"}


def _sources():
    gen = os.path.join(BUILD, "gen")
    os.makedirs(gen, exist_ok=True)
    units = []
    # radix plan 0 for every (precision, length); the alternative plan 1 for FP32 pencils of 32-512 points
    combos = [(tag, ctype, n, 0) for tag, ctype in PRECISIONS.items() for n in LENGTHS]
    combos += [("f32", "float", n, 1) for n in LENGTHS if n >= 32]
    for tag, ctype, n, plan in combos:
        path = os.path.join(gen, f"pass_{tag}_{n}" + (f"_p{plan}" if plan else "") + ".cu")
        text = ('#define GPE_PASS_DEFINITIONS\n#include "gpe_launch.cuh"\n'
                f"GPE_INSTANTIATE_N({ctype}, {n}, {plan})\n")
        if not os.path.isfile(path) or open(path).read() != text:
            with open(path, "w") as fh:
                fh.write(text)
        units.append(path)
    units.append(os.path.join(CSRC, "gpe_engine.cu"))
    units.append(os.path.join(CSRC, "gpe_noalloc.cu"))
    units.append(os.path.join(CSRC, "gpe_probe.cu"))
    units.append(os.path.join(CSRC, "gpe_batch_kernels.cu"))
    units.append(os.path.join(CSRC, "gpe_dropin.cpp"))
    units.append(os.path.join(CSRC, "gpe_snapshots.cpp"))
    return units


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
           [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _compile(src: str, hdr_mtime: float, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.isfile(obj) and os.path.getmtime(obj) > max(os.path.getmtime(src), hdr_mtime):
        return obj
    if src.endswith(".cpp"):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
               "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
    else:
        cmd = ["nvcc", *ARCH, *NVFLAGS, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stderr[-6000:]}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    hdr = max(os.path.getmtime(h) for h in _headers() + [__file__])
    jobs = jobs or max(2, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr, verbose), srcs))
    if os.path.isfile(LIB) and os.path.getmtime(LIB) > max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["nvcc", *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stderr[-6000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
