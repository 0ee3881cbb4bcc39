"""Precision study: FP32 and FP32 + Kahan-compensated velocities against FP64, same scheme.

The orthorhombic layered model of the 320 x 320 x 256 benchmark (same seeded 12-layer table)
resampled to n^3 cells, run for nt steps in each precision on the GPU; every seismogram of the
FP32 runs is compared with the FP64 run's: relative L2 error ||a - ref|| / ||ref|| and relative
peak-amplitude error |max|a| - max|ref|| / max|ref|.

    python -m elanfmt_gb300.precision [--n 256] [--nt 6000] [--out report.json]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import fields as F
from . import inputs as I
from .solver import Solver


def errors(a: np.ndarray, ref: np.ndarray, floor: float = 1e-3) -> dict:
    """Per-trace errors of `a` against `ref`.  A trace whose reference norm is below `floor` times
    the largest trace norm has seen no arrival yet (only the grid's numerical precursor, at the
    rounding level): its relative error has no meaning, so it is counted apart and left out."""
    l2, peak = [], []
    norms = np.linalg.norm(ref, axis=1)
    cut = floor * norms.max() if len(norms) else 0.0
    below = 0
    for r in range(len(ref)):
        n = norms[r]
        pk = np.max(np.abs(ref[r]))
        if n == 0 or pk == 0 or n < cut:
            below += 1
            continue
        l2.append(float(np.linalg.norm(a[r] - ref[r]) / n))
        peak.append(float(abs(np.max(np.abs(a[r])) - pk) / pk))
    l2 = np.array(l2)
    peak = np.array(peak)
    return {"traces": int(len(l2)), "traces_without_arrival": below, "norm_floor": floor,
            "rel_l2_max": float(l2.max()), "rel_l2_median": float(np.median(l2)),
            "rel_l2_mean": float(l2.mean()), "peak_err_max": float(peak.max()),
            "peak_err_median": float(np.median(peak)), "rel_l2_per_trace": [float(v) for v in l2]}


def study(n: int = 256, nt: int = 6000, tune: bool = True) -> dict:
    """The three runs (each form with its autotuned launch setting unless tune is False) and the
    FP32 forms' errors against FP64."""
    m = I.ortho_layered(nx=n, ny=n, nz=n, nt=nt, src=(n // 2, n // 2, n // 2),
                        rec_coords=[int(round(v)) for v in (n * (0.125 + 0.75 * q / 7) for q in range(8))])
    out = {"model": f"orthorhombic layered {n}^3 (12-layer table of the 320x320x256 workload), {nt} steps",
           "receivers": int(len(m.receivers))}
    traces = {}
    for name, prec in (("fp64", F.PREC_F64), ("fp32", F.PREC_F32), ("fp32_kahan", F.PREC_F32_KAHAN)):
        with Solver.from_model(m, precision=prec) as s:
            if tune:
                s.autotune(min(10, nt - 1))
            t = time.perf_counter()
            ms = s.run(nt)
            traces[name] = s.seismograms()
            out[f"{name}_seconds"] = round(time.perf_counter() - t, 3)
            out[f"{name}_gcells"] = round(m.cells * nt / (ms * 1e-3) / 1e9, 2)
    out["fp32_vs_fp64"] = errors(traces["fp32"], traces["fp64"])
    out["fp32_kahan_vs_fp64"] = errors(traces["fp32_kahan"], traces["fp64"])
    out["max_abs_trace"] = float(np.abs(traces["fp64"]).max())
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--nt", type=int, default=6000)
    ap.add_argument("--out", default="")
    args = ap.parse_args()
    res = study(args.n, args.nt)
    short = {k: (v if not isinstance(v, dict) else {kk: vv for kk, vv in v.items() if kk != "rel_l2_per_trace"})
             for k, v in res.items()}
    print(json.dumps(short, indent=1))
    if args.out:
        with open(args.out, "w") as fh:
            json.dump(res, fh)


if __name__ == "__main__":
    main()
