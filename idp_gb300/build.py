"""Builds libidp_gb300.so (the C-ABI library) in-tree with nvcc for sm_103a.

Translation units that must reproduce the reference's FP64 constraint set
and CCD step bit for bit (contact.cu, ccd.cu) are compiled with
--fmad=false; the others keep fused multiply-add. Objects go to
idp_gb300/_build/, the library to idp_gb300/libidp_gb300.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libidp_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unused-function", "-I", INCLUDE]
EXACT_FP64 = {"contact.cu", "ccd.cu", "flow.cu", "dirichlet.cu"}
UNITS = ["prims.cu", "tet.cu", "contact.cu", "barrier.cu", "ccd.cu", "solver.cu", "precond.cu", "vecops.cu",
         "flow.cu", "shell.cu", "shell_elastic.cu", "dirichlet.cu", "surface.cu", "engine.cpp", "server.cpp"]
HEADERS = ["common.cuh", "prims.cuh", "geom.cuh", "grid.cuh", "engine.hpp", "predicates.cuh", "psd.cuh"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _newest_dep():
    deps = [os.path.join(SRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "idp_gb300.h")]
    return max(os.path.getmtime(d) for d in deps)


def _compile(unit, extra=()):
    src = os.path.join(SRC, unit)
    obj = os.path.join(OUT_DIR, unit + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _newest_dep()):
        return obj, None
    flags = list(COMMON) + list(ARCH)
    if unit in EXACT_FP64:
        flags += ["--fmad=false"]
    flags += list(extra)
    lang = ["-x", "cu"]
    cmd = [nvcc()] + lang + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"$ {' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(verbose=False, extra=()):
    """Compile every unit (in parallel) and link the shared library."""
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda u: _compile(u, extra), UNITS))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
