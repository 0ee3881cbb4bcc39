"""Build recipe of the native parts: libewfd.so (CUDA, sm_103a) and the ``ewfd`` executable.

Compiles in-tree (outputs next to this file) with nvcc/gcc directly: a few translation units
built in parallel, one ``-gencode`` for GB300.  The device code is compiled with
``--fmad=false`` (host code: ``-ffp-contract=off``) so that every floating-point operation
rounds on its own, as in the reference's expression order, and host and device code that
share arithmetic agree bit for bit on both x86 and Arm hosts; the kernels are
bandwidth-bound, so the separate multiply and add cost nothing measurable.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", INCLUDE, "-I", CSRC]

LIB = os.path.join(PKG, "libewfd.so")
EXE = os.path.join(PKG, "ewfd")


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}")
    if os.environ.get("EWF_BUILD_VERBOSE"):
        sys.stdout.write(res.stdout)


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def sources() -> list[str]:
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] + [os.path.join(INCLUDE, "ewfd.h")]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libewfd.so and ewfd; returns the library path."""
    srcs = sources()
    if not force and _newer(LIB, srcs) and _newer(EXE, srcs):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    units = [("ewfd.cu", "ewfd.o"), ("ewfd_batch.cu", "ewfd_batch.o"), ("ewfd_band.cu", "ewfd_band.o"), ("ewfd_staged.cu", "ewfd_staged.o"), ("ewf_mlp.cu", "ewf_mlp.o"),
             ("ewfd_post.cu", "ewfd_post.o"), ("ewfd_legacy.cpp", "ewfd_legacy.o")]
    cmds = []
    for src, obj in units:
        extra = ["-x", "cu"] if src.endswith(".cu") else []
        cmds.append([nv, *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", os.path.join(BUILD, obj)])
    if verbose:
        cmds[0].insert(1, "-Xptxas=-v")
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(_run, cmds))
    objs = [os.path.join(BUILD, o) for _, o in units]
    tmp = LIB + ".tmp"
    _run([nv, *ARCH, "-shared", "-o", tmp, *objs, "-Xlinker", "-soname=libewfd.so"])
    os.replace(tmp, LIB)
    cc = shutil.which("gcc") or "cc"
    _run([cc, "-O2", "-Wall", "-I", INCLUDE, os.path.join(CSRC, "ewfd_main.c"), "-L", PKG, "-lewfd",
          "-Wl,-rpath,$ORIGIN", "-o", EXE + ".tmp"])
    os.replace(EXE + ".tmp", EXE)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
