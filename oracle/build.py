"""Build recipe of the test-only checkers under oracle/ (TEST INFRASTRUCTURE ONLY).

* ``libewf_oracle.so`` -- the CPU restatement (ewf_oracle.c), gcc, no FP contraction, OpenMP.
* ``librefkernels.so`` -- the driver-API launcher for the reference's own kernels (refkernels.c).
* ``_ref/*.cubin``     -- the reference solvers' device code compiled from the reference sources
  where they lie (only where the reference tree is present; the cubins then travel with the
  repository copy).  The isotropic (OK4), orthorhombic (ANISO), 9 km (isotropic with edge shear
  moduli), 16 km (the 9 km scheme with linear velocity damping), DC_Earthquake (isotropic
  with per-component weights), the two BC1-free isotropic variants (diff_BC2_OK3, diff_BC_OK2)
  and the FULL scheme (3-D weights, scalar moduli), each with the
  reference's own flags (``-O3``, FMA contraction on: "stock") and with ``--fmad=false``
  ("exact", every operation rounded on its own, which the oracle matches bit for bit).

Nothing here is part of the product.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(HERE, "libewf_oracle.so")
REFK_LIB = os.path.join(HERE, "librefkernels.so")

# where the reference sources lie (only this build step reads them); override with EWF_REFERENCE_ROOT
REFERENCE_ROOT = os.environ.get("EWF_REFERENCE_ROOT", "/root/reference")
REF_SOURCES = {
    "ok4": "src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_OK4_final/FastWaveED_GPU3D_v1.cu",
    "aniso": "src/FastWaveED_GPU3D_v1_9km_station_ANISO/FastWaveED_GPU3D_v1_9kmst_ANISO.cu",
    "iso9km": "src/FastWaveED_GPU3D_v1_9km_station/FastWaveED_GPU3D_v1_9kmst.cu",
    "iso16km": "src/FastWaveED_GPU3D_v1_16km_station/FastWaveED_GPU3D_v1_16kmst.cu",
    "dcq": "src/FastWaveED_GPU3D_v1_DC_Earthquake/FastWaveED_GPU3D_v1.cu",
    # isotropic without BC1, shear modulus 1e-5 on plane 1 (the diff_BC2 scheme)
    "ok3": "src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_diff_BC2_OK3/FastWaveED_GPU3D_v1.cu",
    # the 3-D-weight isotropic form with scalar moduli, without BC1 (the diff_BC scheme)
    "ok2": "src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_diff_BC_OK2/FastWaveED_GPU3D_v1.cu",
    # the same form with BC1 and a separate source kernel
    "full": "src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL/FastBiot_GPU3D_v1.cu",
}
# The grid defines only size the host-side constants of the reference; every kernel takes
# nx, ny, nz as arguments, so one build serves every grid.
REF_DEFINES = ["-DNBX=1", "-DNBY=1", "-DNBZ=1", "-DOVERX=0", "-DOVERY=0", "-DOVERZ=0",
               "-DNPARS1=10", "-DNPARS2=13", "-DNPARS3=12"]


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}")


def _stale(target: str, srcs: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in srcs)


def _nvcc() -> str | None:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def cubin_path(model: str, variant: str) -> str:
    return os.path.join(REF_OUT, f"{model}_{variant}.cubin")


def build_ref_cubins(force: bool = False) -> list[str]:
    """Compile the reference kernels into oracle/_ref/ (no-op where the reference is absent)."""
    nv = _nvcc()
    if not nv or not os.path.isdir(REFERENCE_ROOT):
        return []
    os.makedirs(REF_OUT, exist_ok=True)
    cmds, outs = [], []
    for model, rel in REF_SOURCES.items():
        src = os.path.join(REFERENCE_ROOT, rel)
        for variant, fmad in (("stock", "true"), ("exact", "false")):
            out = cubin_path(model, variant)
            outs.append(out)
            if force or _stale(out, [src]):
                cmds.append([nv, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", f"--fmad={fmad}",
                             "-w", *REF_DEFINES, src, "-o", out])
    with ThreadPoolExecutor(max_workers=max(1, min(8, len(cmds)))) as ex:
        list(ex.map(_run, cmds))
    return outs


def build_oracle(force: bool = False) -> str:
    src = [os.path.join(HERE, "ewf_oracle.c"), os.path.join(HERE, "ewf_oracle_body.h")]
    if force or _stale(ORACLE_LIB, src):
        cc = shutil.which("gcc") or "cc"
        _run([cc, "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
              src[0], "-o", ORACLE_LIB + ".tmp"])
        os.replace(ORACLE_LIB + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


def build_refkernels(force: bool = False) -> str:
    src = [os.path.join(HERE, "refkernels.c")]
    if force or _stale(REFK_LIB, src):
        cc = shutil.which("gcc") or "cc"
        _run([cc, "-O2", "-fPIC", "-shared", src[0], "-o", REFK_LIB + ".tmp", "-ldl"])
        os.replace(REFK_LIB + ".tmp", REFK_LIB)
    return REFK_LIB


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_oracle, force), ex.submit(build_refkernels, force), ex.submit(build_ref_cubins, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("ok")
