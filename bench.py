#!/usr/bin/env python
"""Benchmark of the staggered-grid elastic FDTD time loop (one JSON line on stdout).

Workload (default): the orthorhombic layered model, 320 x 320 x 256 cells, FP32, 4000 time steps,
64 surface receivers x 3 components (seeded synthetic inputs, see elanfmt_gb300/inputs.py).
One bench "step" is one full run of the workload through libewfd.so with the inputs resident in
HBM; `value` = cell-updates per second over the K timed runs (CUDA events on the solver's stream,
max over ranks).  The working set (21 fields, ~2.7 GB in the padded layout) is far larger
than L2, so no flush is needed.

Also reported: `e2e` (the same runs through the C ABI from pinned host buffers, H2D of every
input and D2H of the seismograms inside the timed region), `roofline` (algorithmic bytes of the
dominant kernel / its CUDA-event duration, against MEASURED_PEAKS.json), `cpu_baseline` (the
FP64 C loop of the reference scheme, i.e. the CPU oracle, on the host cores, bounded sample),
`reference_gpu` (the reference's own kernels, compiled from its sources, on the same GPU and
workload), `clocks` (nvidia-smi sampled during the timed region) and `gpu_launches`.

--impl reference times the reference's CPU implementation of the path (the oracle port, FP64,
all host threads) on the same workload and metric, each step a bounded sample of time steps.
Multi-GPU: replicas only (independent runs, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s & % HBM roofline; Green's-fn sets/s surrogate vs FDTD @<=1e-3 L2"
UNIT = "Gcell-updates/s"

# compulsory DRAM bytes per cell-update, FP32 (each state field read+written once, each material
# field read once, separable damping ~0): whole step, and per kernel of the two-kernel step
STEP_BYTES = {"ortho": 120, "iso": 80}
KERNEL_BYTES = {
    "ortho": {"stress": 4 * (3 + 6 + 9 + 6), "velocity": 4 * (6 + 3 + 3 + 3)},
    "iso": {"stress": 4 * (3 + 6 + 2 + 6), "velocity": 4 * (6 + 3 + 3)},
}


ONEPASS_NAMES = ["tile", "band4", "band8", "staged"]  # ewf_set_onepass values, in order
ONEPASS_KERNELS = ["k_step", "k_band", "k_band", "k_staged"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ortho", choices=["ortho", "iso", "batch"])
    ap.add_argument("--nt", type=int, default=0, help="time steps per run (default: the workload's)")
    ap.add_argument("--size", type=str, default="", help="override grid, e.g. 128x128x96 (profiling runs)")
    ap.add_argument("--no-extras", action="store_true", help="skip e2e, cpu baseline, reference_gpu, kernel timing")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--step", default="split", choices=["split", "fused", "wave"],
                    help="step form: two kernels (default), the one-pass kernel or the wavefront launch")
    ap.add_argument("--kchunk", type=int, default=0, help="z-chunk / slab planes (0: autotuned)")
    ap.add_argument("--tile", type=int, default=0, help="CTA tile height in rows, with --kchunk (0: autotuned)")
    ap.add_argument("--l2pf", type=int, default=0, help="velocity kernel's L2 prefetch distance, with --kchunk --tile")
    ap.add_argument("--onepass", default="", choices=["", "tile", "band4", "band8", "staged"],
                    help="one-pass step: its kernel, with --kchunk (default: autotuned)")
    ap.add_argument("--wave-lag", type=int, default=0, help="wavefront lag in %% of the CTAs (0: autotuned)")
    ap.add_argument("--batch-iso", type=int, default=16, help="batch workload: isotropic models beside the 6 MTs")
    ap.add_argument("--no-reference", action="store_true", help="batch workload: skip the reference kernels' runs")
    return ap.parse_args()


def workload(name: str, nt: int, size: str):
    from elanfmt_gb300 import inputs as I

    if name == "ortho":
        nx, ny, nz = (int(v) for v in size.split("x")) if size else (320, 320, 256)
        m = I.ortho_layered(nx=nx, ny=ny, nz=nz, nt=nt or 4000, src=(nx // 2, ny // 2, nz // 2),
                            rec_coords=None if (nx, ny) == (320, 320) else
                            [int(round(v)) for v in (min(nx, ny) * (0.125 + 0.75 * q / 7) for q in range(8))])
        desc = f"orthorhombic layered {nx}x{ny}x{nz}, {m.nt} steps, 12 layers, 15-cell PML, lune MT, Ricker 1.5 Hz"
    else:
        n = int(size.split("x")[0]) if size else 128
        m = I.iso_homogeneous(n=n, nt=nt or 1000)
        desc = f"isotropic homogeneous {n}^3, {m.nt} steps, 10-cell PML, DC MT, Ricker 2 Hz"
    return m, desc


def workload_config(m, desc: str, world: int) -> dict:
    """The `config` of a bench line: what the workload is, the same for both arms."""
    ws = m.cells * 4 * 21  # 9 state + 12 material fields, FP32
    return {"workload": desc, "grid": [m.nx, m.ny, m.nz], "nt": m.nt, "receivers": len(m.receivers),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": ("inputs larger than L2 (working set ~%.1f GB)" % (ws / 1e9)) if ws > 129e6 else
                  ("working set ~%.0f MB, within L2 (no flush between runs)" % (ws / 1e6))}


class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, workload_name: str):
    """DRAM bytes per cell of a kernel from the committed ncu summary (None if absent)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        kv = dict(t.split("=", 1) for t in line.split() if "=" in t)
        if kv.get("kernel") == kernel and kv.get("workload") == workload_name:
            return float(kv["dram_bytes_per_cell"])
    return None


def max_over_ranks(x: float, dist=None) -> float:
    """The slowest rank's value (replicas: every rank runs the whole workload; the job takes as
    long as its slowest replica).  NCCL reduces device tensors, gloo host tensors."""
    if dist is None or not dist.is_initialized():
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(m, seconds: float) -> dict:
    """FP64 C loop of the reference scheme (the CPU oracle) on this host's cores, bounded sample."""
    from elanfmt_gb300 import fields as F
    from oracle import oracle as O

    r = O.Runner(m, F.PREC_F64)
    r.step(1)                       # first touch of the arrays and thread start-up
    t = time.perf_counter()
    r.step(1)
    one = time.perf_counter() - t   # a steady step sizes the sample
    n = max(1, min(m.nt - 2, int(seconds / max(one, 1e-6))))
    t = time.perf_counter()
    r.step(n)
    dt = time.perf_counter() - t
    return {"value": m.cells * n / dt / 1e9, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"{n} time steps of the full {m.nx}x{m.ny}x{m.nz} grid after 2 warm-up steps, FP64, "
                      f"{dt:.1f} s"}


def reference_gpu(m, nsteps: int) -> dict | None:
    """The reference's own kernels (stock build) on the same workload, timed with its own per-
    launch synchronisation (OK4:487-498 / ANISO:521-550)."""
    import copy

    import numpy as np
    import torch

    from elanfmt_gb300 import fields as F
    from elanfmt_gb300.inputs import separable_weights
    from oracle import refrun as R

    if not R.available(m.model, "stock"):
        return None
    mm = copy.copy(m)
    mm.receivers = None
    if m.model == F.MODEL_ORTHO:
        d = m.damping_arrays
        if F.D_W3D not in d:
            mm.damping_arrays = {F.D_W3D: separable_weights(d[F.D_WX], d[F.D_WY], d[F.D_WZ])}
        xs, ys, zs = (int(v) - 1 for v in m.sources[0, 1:4])
        mm.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), xs, ys, zs, 1)
    r = R.RefRunner(mm, "stock")
    try:
        r.run(5)
        torch.cuda.synchronize()
        t = time.perf_counter()
        r.run(nsteps)
        dt = time.perf_counter() - t
    finally:
        r.close()
    return {"value": m.cells * nsteps / dt / 1e9, "unit": UNIT, "steps": nsteps,
            "what": "reference kernels compiled from the reference sources (-O3, sm_103a), launch + sync per kernel"}


def parity_vs_reference(m, form: int) -> dict | None:
    """Every seismogram of a full run of the product against the reference's own kernels (stock
    build, the reference's flags) on the same inputs: relative L2 per trace.  The orthorhombic
    reference hard-codes its moment tensor (ANISO:233-247), so both runs use that tensor at the
    workload's source cell."""
    import copy

    import numpy as np

    from elanfmt_gb300 import fields as F
    from elanfmt_gb300.solver import Solver
    from oracle import refrun as R

    if not R.available(m.model, "stock"):
        return None
    m = copy.copy(m)
    if m.model == F.MODEL_ORTHO:
        xs, ys, zs = (int(v) - 1 for v in m.sources[0, 1:4])
        m.set_moment_tensor(np.array(F.ANISO_LEGACY_MT), xs, ys, zs, 1)
    r = R.RefRunner(m, "stock")
    try:
        r.run(m.nt)
        rt = r.traces.copy()
    finally:
        r.close()
    with Solver.from_model(m, fused=form) as s:
        s.run(m.nt)
        pt = s.seismograms()
    e = R.trace_errors(pt, rt)
    return {"max_rel_l2": float("%.3e" % e["max_rel_l2"]), "median_rel_l2": float("%.3e" % e["median_rel_l2"]),
            "traces": e["traces"], "steps": m.nt, "bar": 1e-4, "pass": bool(e["max_rel_l2"] <= 1e-4 and
                                                                         e["zero_mismatch"] == 0),
            "vs": "reference kernels compiled from the reference sources with its own flags (-O3, sm_103a), "
                  "full run, same inputs" + (" (the ANISO built-in moment tensor)" if m.model == F.MODEL_ORTHO else "")}


def extra_iso(form: int) -> dict:
    """Isotropic homogeneous 128^3, 1000 steps, 8-receiver ring (the plain isotropic workload):
    Gcell-updates/s over full runs with the autotuned setting, the step roofline, and full-run
    seismogram parity against the reference's stock build."""
    from elanfmt_gb300 import fields as F
    from elanfmt_gb300.solver import Solver

    m, desc = workload("iso", 0, "")
    with Solver.from_model(m, fused=form) as s:
        kchunk = s.autotune(20)
        tile = (s.tile(), s.l2_prefetch()) if form == F.STEP_SPLIT else None
        s.reset()
        s.run(m.nt)
        ms = []
        for _ in range(3):
            s.reset()
            ms.append(s.run(m.nt))
    best = statistics.median(ms)
    value = m.cells * m.nt / (best * 1e-3) / 1e9
    peak, kind = peaks()
    return {"workload": desc, "value": round(value, 3), "unit": UNIT, "ms_per_run": round(best, 3), "runs": len(ms),
            "kchunk_autotuned": kchunk,
            **({"tile_y_autotuned": tile[0], "l2_prefetch_autotuned": tile[1]} if tile else {}),
            "step_roofline": {"bytes_per_cell": STEP_BYTES["iso"], "achieved": round(value * STEP_BYTES["iso"], 1),
                              "peak": peak, "unit": "GB/s", "frac": round(value * STEP_BYTES["iso"] / peak, 4),
                              "peak_kind": kind},
            "parity": parity_vs_reference(m, form)}


def solo_seconds(probs, nt: int, tune_steps: int = 6, check=None) -> float:
    """Device seconds of every (problem, RHS) of a batch run alone for nt steps, each with the
    two-kernel step's autotuned z-chunk, tile height and L2 prefetch (tuned once per problem, on
    its first RHS).  check(pid, rhs, traces) sees each solo run's seismograms."""
    from elanfmt_gb300.solver import Solver

    total = 0.0
    for pid, (m, rl) in enumerate(probs):
        setting = None
        for r, (ent, coef) in enumerate(rl):
            with Solver.from_model(m, kchunk=setting[0] if setting else 0) as s:
                s.set_sources(ent, coef)
                if setting is None:
                    setting = (s.autotune(min(tune_steps, nt - 1)), s.tile(), s.l2_prefetch())
                s.set_tile(setting[1])
                s.set_l2_prefetch(setting[2])
                s.run(min(10, nt))
                s.reset()
                total += s.run(nt) * 1e-3
                if check:
                    check(pid, r, s.seismograms())
    return total


def extra_batch(nt: int = 300) -> dict:
    """The batched workload (6 elementary moment tensors on an orthorhombic 256^3 model + 16
    isotropic models 96^3-224^3) on a shortened run of `nt` steps: runs/s of the batched launch
    against each solve launched alone, both on the same steps."""
    from elanfmt_gb300.solver import Batch

    probs = batch_workload(nt)
    runs = sum(len(r) for _, r in probs)
    with Batch(probs) as b:
        b.autotune(5)
        b.run(nt)
        b.reset()
        batch_s = b.run(nt) * 1e-3
        setting = (b.tile(), b.l2_prefetch(), b.launch())
    solo_s = solo_seconds(probs, nt)
    return {"workload": f"6 elementary MTs on orthorhombic 256^3 + 16 isotropic models 96^3-224^3, {nt} steps "
                        f"(the full workload runs 3000)", "runs": runs, "batched_runs_per_s": round(runs / batch_s, 3),
            "solo_runs_per_s": round(runs / solo_s, 3), "speedup_vs_solo": round(solo_s / batch_s, 3),
            "batch_tile_y": setting[0], "batch_l2_prefetch": setting[1],
            "batch_launch": "own launches on parallel branches" if setting[2] else "persistent family launch",
            "solo": "each run alone with its own autotuned z-chunk and tile height"}


def extra_precision(nt: int = 2000) -> dict:
    """The precision study's model (orthorhombic 256^3) on a shortened run of nt steps (the full
    study runs 6000; by step 2000 the direct waves have reached the surface receivers): FP32 and
    FP32 + Kahan against FP64, per-trace relative L2, and the Gcell-updates/s of each form with
    its autotuned setting."""
    from elanfmt_gb300 import precision as P

    r = P.study(n=256, nt=nt)
    return {"workload": r["model"] + " (the full study runs 6000)", "receivers": r["receivers"],
            **{f"{k}_gcell_updates_per_s": r[f"{k}_gcells"] for k in ("fp32", "fp32_kahan", "fp64")},
            **{f"{k}_vs_fp64_rel_l2": {q: r[f"{k}_vs_fp64"][q] for q in ("rel_l2_max", "rel_l2_median", "traces",
                                                                         "traces_without_arrival")}
               for k in ("fp32", "fp32_kahan")}}


def extra_surrogate() -> dict:
    """The learned Green's-function surrogate at the study's network size: inference GF sets/s
    (CUDA events, 4096 queries, forward pass + azimuthal mixing, 1024 samples) next to the
    solver's GF sets/s on the surrogate's 192^3 grid (one source, its 6 elementary runs batched,
    every surface receiver of the study's 12-cell mesh, a 128-step sample scaled to 1024 steps);
    the held-out error is the committed study's."""
    import numpy as np

    from elanfmt_gb300 import fields as F
    from elanfmt_gb300 import surrogate as SG
    from elanfmt_gb300.solver import Batch

    inf = SG.infer_benchmark(nq=4096, nt=1024)
    m = SG.layered_iso(n=192, nt=1024)
    rec_xy = SG.surface_receivers(192, 15, 6)
    rec = np.array([(i, j, 1, c) for i, j in rec_xy for c in (0, 1, 2)], np.int32)
    m.receivers = rec
    rl = []
    for q in range(6):
        mt = np.zeros(6)
        mt[q] = 1.0
        rl.append(F.mt_point_entries(mt, 96, 96, 40))
    sample = 128
    with Batch([(m, rl)]) as b:
        b.run(sample)
        b.reset()
        s_per_src = b.run(sample) * 1e-3 * (1024 / sample)
    fdtd = len(rec_xy) / s_per_src
    out = {"network": inf["network"], "surrogate_gf_sets_per_s": round(inf["gf_sets_per_s"], 1),
           "fdtd_gf_sets_per_s": round(fdtd, 1), "ratio": round(inf["gf_sets_per_s"] / fdtd, 1),
           "fdtd_sample": f"{sample} of 1024 steps, 192^3, 6 RHS batched, {len(rec_xy)} receivers, scaled linearly"}
    study = os.path.join(ROOT, "profiles", "surrogate_study.json")
    if os.path.exists(study):
        res = json.load(open(study))
        out["held_out_error"] = {k: res.get(k) for k in ("median_rel_l2", "p90_rel_l2", "served_at_1e-3", "workload")}
    return out


def main():
    args = parse()
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    if args.impl == "reference":
        if rank != 0:
            return
        return main_reference(args)
    if args.workload == "batch":
        return main_batch(args)

    from elanfmt_gb300 import fields as F
    from elanfmt_gb300.solver import Solver

    torch.cuda.set_device(local)
    m, desc = workload(args.workload, args.nt, args.size)
    nt = m.nt
    form = {"split": F.STEP_SPLIT, "fused": F.STEP_FUSED, "wave": F.STEP_WAVE}[args.step]
    s = Solver.from_model(m, fused=form, kchunk=args.kchunk)
    # the library's autotuner (z-chunk; the wavefront lag too) unless both are given
    kchunk = args.kchunk if args.kchunk and (form != F.STEP_WAVE or args.wave_lag) else s.autotune(30)
    if form == F.STEP_WAVE and args.wave_lag:
        s.set_wave(args.wave_lag)
    if form == F.STEP_SPLIT and args.kchunk and args.tile:
        s.set_tile(args.tile)
        s.set_l2_prefetch(args.l2pf)
    if form == F.STEP_FUSED and args.kchunk and args.onepass:
        s.set_onepass(ONEPASS_NAMES.index(args.onepass))

    for _ in range(args.warmup):
        s.reset()
        s.run(nt)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = Clocks(local)
    clk.start()
    ms = []
    for _ in range(args.steps):
        s.reset()
        ms.append(s.run(nt))
    torch.cuda.synchronize()
    clocks = clk.stop()
    total_ms = max_over_ranks(sum(ms), dist)
    units = m.cells * nt * args.steps * world
    value = units / (total_ms * 1e-3) / 1e9
    launches = s.launches_per_step() * nt * args.steps

    peak, peak_kind = peaks()
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": workload_config(m, desc, world),
        "tuning": {"step": args.step, "kchunk_autotuned": kchunk,
                   **({"tile_y_autotuned": s.tile(), "l2_prefetch_autotuned": s.l2_prefetch()}
                      if form == F.STEP_SPLIT else {}),
                   **({"wave_lag_pct": s.wave_lag()} if form == F.STEP_WAVE else {}),
                   **({"onepass_kernel": ONEPASS_NAMES[s.onepass()]} if form == F.STEP_FUSED else {})},
        "gpu_launches": launches,
    }
    step_frac = value * STEP_BYTES[args.workload] / peak
    out["step_roofline"] = {"bytes_per_cell": STEP_BYTES[args.workload], "achieved": round(value * STEP_BYTES[args.workload], 1),
                            "peak": peak, "unit": "GB/s", "frac": round(step_frac, 4), "peak_kind": peak_kind}
    if clocks:
        out["clocks"] = clocks

    if not args.no_extras and rank == 0:
        # per-kernel CUDA-event timing on the solver's stream
        s.reset()
        kt = s.time_kernels(min(200, nt))
        if form == F.STEP_SPLIT:
            kb = KERNEL_BYTES[args.workload]
            names = {"stress": "k_stress", "velocity": "k_velocity"}
        else:  # one kernel does the whole step: its compulsory bytes are the one-pass step's
            kb = {"stress": STEP_BYTES[args.workload]}
            names = {"stress": "k_wave" if form == F.STEP_WAVE else ONEPASS_KERNELS[s.onepass()]}
        kernels = {}
        for k in kb:
            achieved = kb[k] * m.cells / (kt[k] * 1e-3) / 1e9
            kernels[k] = {"ms": round(kt[k], 4), "bytes_per_cell": kb[k], "achieved_gbs": round(achieved, 1),
                          "frac": round(achieved / peak, 4)}
        dom = max(kb, key=lambda k: kt[k])
        tr = ncu_traffic(names[dom], args.workload)
        out["roofline"] = {"kernel": names[dom], "bound": "hbm", "achieved": kernels[dom]["achieved_gbs"],
                           "peak": peak, "unit": "GB/s", "frac": kernels[dom]["frac"],
                           "traffic": None if tr is None else round(tr * m.cells),
                           "algorithmic_bytes": kb[dom] * m.cells, "peak_kind": peak_kind}
        out["kernels"] = kernels | {"inject_ms": round(kt["inject"], 4), "record_ms": round(kt["record"], 4)}
        out["e2e"] = e2e(s, m, args.steps)
        out["reference_gpu"] = reference_gpu(m, 200 if m.cells > 10_000_000 else 500)
        out["cpu_baseline"] = cpu_baseline(m, args.cpu_seconds)
    s.close()
    if not args.no_extras and rank == 0:
        out["parity"] = parity_vs_reference(m, form)
        if args.workload == "ortho" and not args.size and not args.nt:
            # the other workloads, bounded (about a minute together)
            for key, fn in (("iso", lambda: extra_iso(form)), ("precision", extra_precision), ("batch", extra_batch),
                            ("surrogate", extra_surrogate)):
                t = time.perf_counter()
                try:
                    out[key] = fn()
                except Exception as e:  # an extra leg never voids the headline line
                    out[key] = {"error": f"{type(e).__name__}: {e}"[:300]}
                out[key]["bench_seconds"] = round(time.perf_counter() - t, 1)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def e2e(s, m, steps: int) -> dict:
    """Through the C ABI with host buffers: every input H2D from pinned memory, the full run, the
    seismograms D2H -- all inside the timed region."""
    import numpy as np
    import torch

    pinned = []
    for fid, arr in list(m.materials.items()) + list(m.damping_arrays.items()):
        t = torch.from_numpy(np.ascontiguousarray(arr)).pin_memory()
        pinned.append((fid, t))
    stf = torch.from_numpy(np.ascontiguousarray(m.stf, np.float64)).pin_memory()
    h2d = sum(t.numel() * t.element_size() for _, t in pinned) + stf.numel() * 8 + m.sources.size * 4 + \
        m.source_coef.size * 8 + m.receivers.size * 4
    trace = torch.empty((len(m.receivers), m.nt), dtype=torch.float64).pin_memory()
    d2h = trace.numel() * 8
    n = max(1, min(steps, 2))
    times = []
    for _ in range(n):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for fid, t in pinned:
            s.set_field_ptr(fid, t.data_ptr(), t.numel(), t.element_size())
        s._lib.ewf_set_stf(s._h, stf.data_ptr(), stf.numel())
        s.set_sources(m.sources, m.source_coef)
        s.set_receivers(m.receivers)
        s.reset()
        s.run(m.nt)
        s._lib.ewf_get_seismograms(s._h, trace.data_ptr(), trace.numel())
        t1 = time.perf_counter()
        times.append(t1 - t0)
    best = statistics.median(times)
    return {"value": round(m.cells * m.nt / best / 1e9, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "runs": n, "seconds_per_step": round(best, 4)}


def batch_workload(nt: int = 3000, n_ortho: int = 256, n_iso: int = 16, seed: int = 4):
    """6 unit elementary moment tensors on one orthorhombic layered n_ortho^3 model, plus n_iso
    isotropic models with seeded sizes uniform in 96^3..224^3 and per-model source depth
    uniform in (0.25, 0.75) nz."""
    import numpy as np

    from elanfmt_gb300 import fields as F
    from elanfmt_gb300 import inputs as I

    mo = I.ortho_layered(nx=n_ortho, ny=n_ortho, nz=n_ortho, nt=nt, src=(n_ortho // 2,) * 3,
                         rec_coords=[int(round(v)) for v in (n_ortho * (0.125 + 0.75 * q / 7) for q in range(8))])
    xs, ys, zs = (int(v) - 1 for v in mo.sources[0, 1:4])
    rhs = []
    for q in range(6):  # Mxx, Myy, Mzz, Mxy, Mxz, Myz
        mt = np.zeros(6)
        mt[q] = 1.0
        rhs.append(F.mt_entries(mt, xs, ys, zs, 1))
    probs = [(mo, rhs)]
    rng = np.random.default_rng(seed)
    for _ in range(n_iso):
        n = int(rng.integers(96, 225))
        m = I.iso_homogeneous(n=n, nt=nt)
        depth = int(rng.uniform(0.25, 0.75) * n)
        c = n // 2
        ent, coef = F.mt_entries(I.mt_strike_dip_rake(30, 60, 90), c - 1, c - 1, depth - 1, 0)
        probs.append((m, [(ent, coef)]))
    return probs


def main_batch(args):
    """Config 4: runs/s of the batched launch against launching each solve alone."""
    import numpy as np
    import torch

    from elanfmt_gb300.solver import Batch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    nt = args.nt or 3000
    n_ortho = int(args.size.split("x")[0]) if args.size else 256
    probs = batch_workload(nt, n_ortho=n_ortho, n_iso=args.batch_iso)
    runs = sum(len(r) for _, r in probs)
    cell_updates = sum(m.cells * len(r) for m, r in probs) * nt
    with Batch(probs, kchunk=args.kchunk) as b:
        if args.kchunk and args.tile:  # a fixed setting (profiling runs)
            k = args.kchunk
            b.set_tile(args.tile)
            b.set_l2_prefetch(args.l2pf)
        else:
            k = b.autotune(10)
        tile = b.tile()
        l2pf = b.l2_prefetch()
        own = b.launch()
        clk = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
        clk.start()
        ms_batch = [b.run(nt)]
        for _ in range(max(0, args.steps - 1)):
            b.reset()
            ms_batch.append(b.run(nt))
        clocks = clk.stop()
        tr0 = b.seismograms(0, 0)
    batch_s = min(ms_batch) * 1e-3

    def check(pid, r, traces):
        if pid == 0 and r == 0:
            assert np.array_equal(traces, tr0), "batched and solo traces differ"

    solo_s = solo_seconds(probs, nt, check=check)
    out = {"metric": "runs/s (batched launch vs each solve alone)", "value": round(runs / batch_s, 4),
           "unit": "runs/s", "n_gpus": 1, "steps": len(ms_batch), "higher_is_better": True,
           "solo_runs_per_s": round(runs / solo_s, 4), "speedup_vs_solo": round(solo_s / batch_s, 3),
           "solo": "each run alone with its own autotuned z-chunk and tile height",
           "batched_gcell_updates_per_s": round(cell_updates / batch_s / 1e9, 2),
           "solo_gcell_updates_per_s": round(cell_updates / solo_s / 1e9, 2),
           "kchunk_autotuned": k, "tile_y_autotuned": tile, "l2_prefetch_autotuned": l2pf,
           "launch_autotuned": "own launches on parallel branches" if own else "persistent family launch", "dtype": "f32",
           "data": "synthetic (seeded)",
           "config": {"workload": f"6 elementary MTs on orthorhombic {n_ortho}^3 + {args.batch_iso} isotropic models "
                                  f"96^3-224^3, {nt} steps",
                      "runs": runs, "cell_updates": cell_updates}}
    if clocks:
        out["clocks"] = clocks
    # the reference's own kernels, one run at a time with their launch + synchronise pattern:
    # each problem's per-run rate over a bounded sample of steps, summed over the runs
    ref_s, rates = (None if args.no_reference else 0.0), []
    for m, rl in (probs if ref_s is not None else []):
        r = reference_gpu(m, 100)
        if r is None:
            ref_s = None
            break
        rates.append(round(r["value"], 2))
        ref_s += m.cells * nt * len(rl) / (r["value"] * 1e9)
    if ref_s:
        out["reference_kernels"] = {"runs_per_s": round(runs / ref_s, 4), "speedup_of_batch": round(ref_s / batch_s, 3),
                                    "gcell_updates_per_s_per_problem": rates,
                                    "what": "reference kernels (stock build), each run alone, 100-step samples"}
    print(json.dumps(out), flush=True)


def main_reference(args):
    """The reference's CPU implementation of the path: the FP64 C loop of the reference scheme
    (oracle port) on all host threads; each bench step is a bounded sample of time steps."""
    from oracle import oracle as O

    from elanfmt_gb300 import fields as F

    m, desc = workload(args.workload, args.nt, args.size)
    r = O.Runner(m, F.PREC_F64)
    t = time.perf_counter()
    r.step(1)
    one = time.perf_counter() - t
    per = max(1, min(20, int(6.0 / max(one, 1e-6)), m.nt - 2))  # a sample never runs past nt
    for _ in range(args.warmup):
        r.step(per) if r.state.it + per < m.nt else None
    times = []
    for _ in range(args.steps):
        if r.state.it + per >= m.nt:
            r = O.Runner(m, F.PREC_F64)
        t = time.perf_counter()
        r.step(per)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = m.cells * per * args.steps / total / 1e9
    sample = f"{per} time steps of the full {m.nx}x{m.ny}x{m.nz} grid per bench step, FP64"
    # n_gpus mirrors the launch (--gpus); the work itself runs on rank 0's host cores (cpu_baseline)
    out = {"impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded)", "config": workload_config(m, desc, args.gpus),
           "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": O.num_threads(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "gpu_launches": 0}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
