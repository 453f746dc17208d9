"""Recipe that builds the reference libcugpe engine as a parity oracle.

TEST INFRASTRUCTURE ONLY: nothing in the product imports or links this.

The reference engine (KKobuszewski/libcugpe, directory ``dev/``) is a
compile-time-configured CUDA library: lattice ``NX/NY/NZ`` and the functional
``INTERACTIONS`` are preprocessor macros (dev/Makefile:2-8, 44-46).  Its
sources need five mechanical edits to compile with nvcc 13 / gcc 13:

1. C99 ``double complex`` is not valid C++: ``cplx`` becomes
   ``std::complex<double>`` (dev/gpe_complex.cuh:36).
2. ``cexp/creal/cimag`` and ``I`` become ``std::exp/real/imag`` and complex
   constructors (dev/gpe_engine.cu:178-180, 190-213, 239-274).
3. ``#include <complex.h>`` is dropped (dev/gpe_engine.h:36,
   dev/gpe_engine.cu:26, dev/gpe_engine.cuh:36).
4. Malformed ``#pragma message`` lines are fixed
   (dev/gpe_user_defined.h:110, dev/gpe_engine.cu:93,95).
5. cuFFT enums removed since CUDA 7 (``CUFFT_INCOMPLETE_PARAMETER_LIST``,
   ``CUFFT_PARSE_ERROR``, ``CUFFT_LICENSE_ERROR``) are defined in a shim
   (used at dev/gpe_engine.h:181-186, 228-233).

Step ``prepare`` (needs the reference checkout) writes the edited copies to
``oracle/_ref/src`` (git-ignored, never committed).  Step ``build`` compiles
``oracle/ref_runner.cu`` (a driver written for this project) against those
copies, one binary per ``(nx, ny, nz, interactions)`` into ``oracle/_ref/bin``.
``build`` works without the reference checkout as long as ``oracle/_ref/src``
exists, so the edited copies can be compiled on a machine that only received
this working tree.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_root() -> str:
    """The reference checkout this recipe reads: $GPE_REFERENCE_ROOT, else the path of the read-only
    checkout on the build machine.  On machines without it (the GPU machine), `build` compiles the edited
    copies already written to oracle/_ref/src."""
    return os.environ.get("GPE_REFERENCE_ROOT", "") or "/root/reference"


REF_ROOT = _reference_root()
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
BIN = os.path.join(OUT, "bin")

FILES = ["gpe_engine.cu", "gpe_engine.h", "gpe_engine.cuh", "gpe_complex.cuh",
         "gpe_user_defined.h", "gpe_timing.h", "reductions.cu", "reductions.cuh"]

SHIM = """// compatibility shim for cuFFT enums removed after CUDA 7
#pragma once
#include <cufft.h>
#define CUFFT_INCOMPLETE_PARAMETER_LIST ((cufftResult)0xA)
#define CUFFT_PARSE_ERROR ((cufftResult)0xC)
#define CUFFT_LICENSE_ERROR ((cufftResult)0xF)
"""


def _edit(name: str, text: str) -> str:
    text = text.replace("#include <complex.h>      // not std::complex!", "")
    if name == "gpe_complex.cuh":
        text = text.replace("typedef double complex cplx;", "typedef std::complex<double> cplx;")
        text = text.replace("#include <cuComplex.h>", "#include <cuComplex.h>\n#include <complex>")
    if name == "gpe_engine.cu":
        text = text.replace("cplx c1=GAMMA*0.5*dt + I*0.0;", "cplx c1(GAMMA*0.5*dt, 0.0);")
        text = text.replace("cplx c2=-1.0*beta + I*alpha;", "cplx c2(-1.0*beta, alpha);")
        text = re.sub(r"\bcexp\(", "std::exp(", text)
        text = re.sub(r"\bcreal\(", "std::real(", text)
        text = re.sub(r"\bcimag\(", "std::imag(", text)
        text = text.replace('#pragma message (__FILE__ ":" __LINE__ "Setting MAX USER PARAMS: " xstr(MAX_USER_PARAMS))', "")
        text = text.replace('#pragma message (__FILE__ ":" __LINE__ " MAX USER PARAMS: " xstr(MAX_USER_PARAMS))', "")
    if name == "gpe_user_defined.h":
        text = text.replace('#pragma message ()"Compiling for unitary Fermi gas")',
                            '#pragma message ("Compiling for unitary Fermi gas")')
    return text


def prepare() -> bool:
    dev = os.path.join(REF_ROOT, "dev") if REF_ROOT else ""
    if not dev or not os.path.isdir(dev):
        return os.path.isfile(os.path.join(SRC, "gpe_engine.cu"))
    os.makedirs(SRC, exist_ok=True)
    for f in FILES:
        with open(os.path.join(dev, f), "r", encoding="latin-1") as fh:
            text = fh.read()
        with open(os.path.join(SRC, f), "w", encoding="latin-1") as fh:
            fh.write(_edit(f, text))
    with open(os.path.join(SRC, "cufft_compat.h"), "w") as fh:
        fh.write(SHIM)
    return True


def binary_name(nx: int, ny: int, nz: int, inter: int, vext: int = 0) -> str:
    return os.path.join(BIN, f"ref_{nx}x{ny}x{nz}_i{inter}" + (f"_v{vext}" if vext else ""))


def build_one(nx: int, ny: int, nz: int, inter: int, arch: str = "103a", vext: int = 0) -> str:
    """One reference binary for this lattice and functional; `vext` selects the reference's external
    potential (0 harmonic trap, 1 Woods-Saxon tube: dev/gpe_user_defined.h:478-558)."""
    out = binary_name(nx, ny, nz, inter, vext)
    runner = os.path.join(HERE, "ref_runner.cpp")
    srcs = [os.path.join(SRC, "gpe_engine.cu"), os.path.join(SRC, "reductions.cu"), runner]
    if os.path.isfile(out) and all(os.path.getmtime(out) > os.path.getmtime(s) for s in srcs):
        return out
    os.makedirs(BIN, exist_ok=True)
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["nvcc", "-O3", "-rdc=true", f"-gencode=arch=compute_{arch},code=sm_{arch}",
           "-w", "-include", os.path.join(SRC, "cufft_compat.h"), "-I", SRC,
           f"-DNX={nx}", f"-DNY={ny}", f"-DNZ={nz}", f"-DINTERACTIONS={inter}", f"-DVEXT={vext}",
           *srcs, "-lcufft", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    os.replace(tmp, out)
    return out


# lattices used by the parity tests and the golden-vector generator
DEFAULT_CONFIGS = [
    (16, 16, 16, -1), (32, 16, 8, -1), (16, 16, 16, 0), (8, 32, 16, 0),
    (64, 64, 64, -1), (32, 32, 32, 0), (128, 128, 128, 0),
]


def build(configs=None, jobs: int = 8) -> list[str]:
    if not prepare():
        raise FileNotFoundError("reference sources unavailable (neither the checkout nor oracle/_ref/src)")
    configs = configs or DEFAULT_CONFIGS
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        return list(ex.map(lambda c: build_one(*c), configs))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "prepare":
        print("prepared" if prepare() else "unavailable")
    else:
        for p in build():
            print(p)
