"""Builds libgpe_gb300.so in-tree for sm_103a (GB300).

The fused pass kernel is instantiated in one generated translation unit per
(precision, pencil length, radix plan), compiled in parallel, then linked with
the engine and the drop-in API into ``libcugpe_gb300/_lib/libgpe_gb300.so``.

A library with user hooks (``include/gpe_user_defined.h`` or a copy edited by
the user) is built beside it under its own name:

    python -m libcugpe_gb300.build --hooks my_hooks.h --name mine -DVEXT=1

gives ``libcugpe_gb300/_lib/libgpe_gb300_mine.so``: the same C ABI and drop-in
API, with the pass kernels calling the header's gpe_external_potential,
gpe_dEDFdn, gpe_EDF and gpe_modify_psi.  ``--lengths 16,32`` and
``--precisions f64`` restrict the compiled pencil lengths and precisions (the
others refuse to run) and ``--no-batch`` leaves out the batched solver, which
keeps a library for small test lattices quick to build.
"""
from __future__ import annotations

import argparse
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


def library_path(name: str | None = None) -> str:
    return LIB if not name else os.path.join(LIBDIR, f"libgpe_gb300_{name}.so")


def _sources(build_dir, lengths, precisions, batch=True):
    gen = os.path.join(build_dir, "gen")
    os.makedirs(gen, exist_ok=True)
    units = []
    # radix plan 0 for every (precision, length); the alternative plan 1 for FP32 pencils of 32-512 points
    every = [(tag, ctype, n, 0) for tag, ctype in PRECISIONS.items() for n in LENGTHS]
    every += [("f32", "float", n, 1) for n in LENGTHS if n >= 32]
    stubs = []
    for tag, ctype, n, plan in every:
        if n not in lengths or tag not in precisions:
            stubs.append(f"GPE_INSTANTIATE_N({ctype}, {n}, {plan})\n")
            continue
        path = os.path.join(gen, f"pass_{tag}_{n}" + (f"_p{plan}" if plan else "") + ".cu")
        text = ('#define GPE_PASS_DEFINITIONS\n#include "gpe_launch.cuh"\n'
                f"GPE_INSTANTIATE_N({ctype}, {n}, {plan})\n")
        _write_if_changed(path, text)
        units.append(path)
    if stubs:
        path = os.path.join(gen, "pass_stubs.cu")
        _write_if_changed(path, '#define GPE_PASS_STUBS\n#include "gpe_launch.cuh"\n' + "".join(stubs))
        units.append(path)
    # batched passes (FP32): one unit per (axis, radix plan), or stubs that refuse them
    if batch:
        for ax in ("X", "Y", "Z"):
            for plan in (0, 1):
                path = os.path.join(gen, f"batch_{ax.lower()}_p{plan}.cu")
                _write_if_changed(path, '#define GPE_BATCH_DEFINITIONS\n#include "gpe_batch_kernels.cuh"\n'
                                        f"GPE_INSTANTIATE_BATCH(gpe::AX_{ax}, {plan})\n")
                units.append(path)
    else:
        path = os.path.join(gen, "batch_stubs.cu")
        _write_if_changed(path, '#define GPE_BATCH_STUBS\n#include "gpe_batch_kernels.cuh"\n' + "".join(
            f"GPE_INSTANTIATE_BATCH(gpe::AX_{ax}, {plan})\n" for ax in ("X", "Y", "Z") for plan in (0, 1)))
        units.append(path)
    for f in ("gpe_engine.cu", "gpe_plane.cu", "gpe_noalloc.cu", "gpe_probe.cu", "gpe_batch_dispatch.cu",
              "gpe_dropin.cpp", "gpe_snapshots.cpp"):
        units.append(os.path.join(CSRC, f))
    return units


def _write_if_changed(path, text):
    if not os.path.isfile(path) or open(path).read() != text:
        with open(path, "w") as fh:
            fh.write(text)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
           [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _compile(src: str, build_dir: str, extra: list, dep_mtime: float, verbose: bool) -> str:
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    if os.path.isfile(obj) and os.path.getmtime(obj) > max(os.path.getmtime(src), dep_mtime):
        return obj
    if src.endswith(".cpp"):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
               "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
    else:
        cmd = ["nvcc", *ARCH, *NVFLAGS, *extra, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stderr[-6000:]}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(jobs: int | None = None, verbose: bool = False, hooks: str | None = None, name: str | None = None,
          defines: tuple = (), lengths=None, precisions=None, batch: bool = True) -> str:
    """Builds the library and returns its path.  `hooks`: a user hook header (then `name` is required
    and names the library); `defines`: extra preprocessor definitions ("VEXT=1", ...) for the device
    code; `lengths` / `precisions`: compile only these pencil lengths / precisions ("f64", "f32");
    `batch`: compile the batched solver's kernels (else it refuses to run)."""
    if hooks and not name:
        raise ValueError("a hook library needs a name")
    if name and not name.replace("_", "").isalnum():
        raise ValueError(f"library name {name!r}: letters, digits and '_' only")
    lengths = list(lengths) if lengths else LENGTHS
    precisions = list(precisions) if precisions else list(PRECISIONS)
    build_dir = os.path.join(BUILD, f"lib_{name}") if name else BUILD
    lib = library_path(name)
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = [f"-D{d}" for d in defines]
    deps = _headers() + [__file__, os.path.join(CSRC, "exports.map")]
    if hooks:
        hooks = os.path.abspath(hooks)
        if not os.path.isfile(hooks):
            raise FileNotFoundError(hooks)
        extra.append(f'-DGPE_USER_HOOKS="{hooks}"')
        deps.append(hooks)
    # a change of hook header, definitions or subset rebuilds everything
    stamp = os.path.join(build_dir, "options.txt")
    _write_if_changed(stamp, repr((hooks, sorted(defines), lengths, precisions, batch)))
    deps.append(stamp)
    dep_mtime = max(os.path.getmtime(h) for h in deps)
    srcs = _sources(build_dir, lengths, precisions, batch)
    jobs = jobs or max(2, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, build_dir, extra, dep_mtime, verbose), srcs))
    if os.path.isfile(lib) and os.path.getmtime(lib) > max(os.path.getmtime(o) for o in objs):
        return lib
    tmp = lib + f".tmp{os.getpid()}"
    cmd = ["nvcc", *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart",
           "-Xlinker", "--version-script=" + os.path.join(CSRC, "exports.map")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stderr[-6000:]}")
    os.replace(tmp, lib)
    return lib


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--hooks", help="user hook header (a copy of include/gpe_user_defined.h)")
    ap.add_argument("--name", help="library name: libgpe_gb300_<name>.so")
    ap.add_argument("-D", dest="defines", action="append", default=[], help="preprocessor definition, e.g. -DVEXT=1")
    ap.add_argument("--lengths", help="pencil lengths to compile, e.g. 16,32 (default: all)")
    ap.add_argument("--precisions", help="f64, f32 or f64,f32 (default: both)")
    ap.add_argument("--no-batch", action="store_true", help="leave out the batched solver's kernels")
    ap.add_argument("-v", dest="verbose", action="store_true", help="print ptxas register and spill reports")
    args = ap.parse_args(argv)
    print(build(verbose=args.verbose, hooks=args.hooks, name=args.name, defines=tuple(args.defines),
                lengths=[int(x) for x in args.lengths.split(",")] if args.lengths else None,
                precisions=args.precisions.split(",") if args.precisions else None, batch=not args.no_batch))


if __name__ == "__main__":
    main()
