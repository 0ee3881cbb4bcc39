"""Generates the golden fixtures tests/golden/*.npz from the reference's own kernels.

Run on a machine with a CUDA GPU, from the repository root, after oracle/build.py has compiled
the reference sources into oracle/_ref/*.cubin:

    python tests/golden/make_golden.py [out_dir] [case ...]

For each small seeded case below it replays the reference's time loop with the reference's
kernels (oracle/refrun.py) in both builds -- "exact" (--fmad=false) and "stock" (-O3 with FMA
contraction, the reference's own flags) -- and stores the 9 state fields, the receiver traces
and a SHA-256 of the generated inputs (so a drifting input generator is detected, not
silently compared).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from elanfmt_gb300 import fields as F  # noqa: E402
from elanfmt_gb300 import inputs as I  # noqa: E402


def case_ok4():
    m = I.random_small(F.MODEL_ISO, 14, 16, 12, nt=40, seed=101)
    m.set_moment_tensor(np.array([0.5, -1.0, 0.3, 0.2, 1.0, 0.8]), 4, 5, 3, 0)
    return m


def case_ok4_surface():
    m = I.random_small(F.MODEL_ISO, 14, 16, 12, nt=40, seed=103)
    m.set_moment_tensor(np.array([0.1, 0.2, -0.3, 0.9, 1.1, -0.7]), 5, 5, 1, 0)
    return m


def case_aniso():
    m = I.random_small(F.MODEL_ORTHO, 14, 16, 12, nt=40, seed=102, damping=F.DAMP_W3D)
    m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), 5, 6, 3, 1)
    return m


def case_aniso_surface():
    m = I.random_small(F.MODEL_ORTHO, 14, 16, 12, nt=40, seed=104, damping=F.DAMP_W3D)
    m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), 5, 6, 0, 1)
    return m


def case_iso9km():
    m = I.random_small(F.MODEL_ISO_HET, 14, 16, 12, nt=40, seed=105, damping=F.DAMP_W3D)
    m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), 5, 6, 3, 1)
    return m


def case_iso9km_surface():
    m = I.random_small(F.MODEL_ISO_HET, 14, 16, 12, nt=40, seed=106, damping=F.DAMP_W3D)
    m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), 5, 6, 0, 1)
    return m


def case_iso16km():
    m = I.random_small(F.MODEL_ISO_HET, 14, 16, 12, nt=40, seed=107, damping=F.DAMP_W3D)
    m.set_moment_tensor(np.array(F.ISO16KM_LEGACY_MT), 5, 6, 3, 1)
    m.vdamp = F.VDAMP_16KM
    return m


def case_dcq():
    m = I.random_small(F.MODEL_ISO, 14, 16, 12, nt=40, seed=108, damping=F.DAMP_PERCOMP)
    m.set_moment_tensor(np.array(F.DCQ_LEGACY_MT), 5, 6, 3, 1)
    return m


CASES = {"ok4": case_ok4, "ok4_surface": case_ok4_surface, "aniso": case_aniso, "aniso_surface": case_aniso_surface,
         "iso9km": case_iso9km, "iso9km_surface": case_iso9km_surface, "iso16km": case_iso16km, "dcq": case_dcq}


def input_digest(m) -> str:
    h = hashlib.sha256()
    for d in (m.materials, m.damping_arrays):
        for k in sorted(d):
            h.update(np.ascontiguousarray(d[k]).tobytes())
    for a in (m.sources, m.source_coef, m.stf, m.receivers):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(np.array([m.dx, m.dy, m.dz, m.dt, m.c66, m.bx, m.by, m.bz]).tobytes())
    if getattr(m, "vdamp", 0.0):
        h.update(np.array([m.vdamp]).tobytes())
    if m.damping == F.DAMP_PERCOMP:
        h.update(np.array([m.c44, m.c55]).tobytes())
    return h.hexdigest()


def main(out_dir: str, only=()) -> None:
    from oracle import refrun as R

    os.makedirs(out_dir, exist_ok=True)
    for name, make in CASES.items():
        if only and name not in only:
            continue
        m = make()
        out = {"digest": np.array(input_digest(m)), "nsteps": np.array(m.nt)}
        for variant in ("exact", "stock"):
            r = R.RefRunner(m, variant)
            r.run(m.nt)
            for q, f in enumerate(r.fields()):
                out[f"{variant}_{F.STATE_NAMES[q]}"] = f
            out[f"{variant}_traces"] = r.traces.copy()
            r.close()
        path = os.path.join(out_dir, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"), tuple(sys.argv[2:]))
