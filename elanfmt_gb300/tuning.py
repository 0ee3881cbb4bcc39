"""Cache of the autotuner's choices (JSON), so a workload is timed once per GPU model.

The library's autotuner (`ewf_autotune`, `ewf_batch_autotune`) times the step for z-chunks of
4..64 planes and, for the two-kernel step, CTA tile heights of 4, 8 and 16 rows.  The best
setting depends on the GPU, the scheme (model, damping, precision, step form) and the grid, not
on the inputs' values, so it is stored under that key (the wavefront form's lag is re-tuned by
`ewf_autotune` when a handle needs it):

    from elanfmt_gb300 import tuning
    k = tuning.kchunk_for(model, precision=F.PREC_F32)      # cached, or tuned once and stored
    with Solver.from_model(model, kchunk=k) as s: ...

    k, ty, pf = tuning.split_setting_for(model)             # z-chunk, tile height, L2 prefetch
    with Solver.from_model(model, kchunk=k) as s:
        s.set_tile(ty)
        s.set_l2_prefetch(pf)

The cache file defaults to $EWF_TUNING_CACHE or ~/.cache/elanfmt_gb300/kchunk.json.
"""
from __future__ import annotations

import json
import os
import tempfile

from . import fields as F


def cache_path() -> str:
    return os.environ.get("EWF_TUNING_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "elanfmt_gb300",
                                                              "kchunk.json")


FORM_NAMES = {F.STEP_SPLIT: "split", F.STEP_FUSED: "fused", F.STEP_WAVE: "wave"}


def key(device_name: str, m, precision: int, form: int) -> str:
    return (f"{device_name}|model{m.model}|damp{m.damping}|prec{precision}|{FORM_NAMES[int(form)]}|"
            f"{m.nx}x{m.ny}x{m.nz}")


def load(path: str | None = None) -> dict:
    p = path or cache_path()
    try:
        with open(p) as fh:
            data = json.load(fh)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store(k: str, value, path: str | None = None) -> None:
    """Adds one entry (an int, or a list of ints); the file is replaced atomically so concurrent
    writers never leave it torn."""
    p = path or cache_path()
    data = load(p)
    data[k] = [int(v) for v in value] if isinstance(value, (list, tuple)) else int(value)
    os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=os.path.dirname(p) or ".", suffix=".tmp")
    with os.fdopen(fd, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, p)


def kchunk_for(m, precision: int = F.PREC_F32, fused: int = F.STEP_SPLIT, nsteps: int = 30, path: str | None = None,
               device_name: str | None = None, tune=None) -> int:
    """The cached z-chunk for this workload shape and step form (F.STEP_*), or the autotuner's
    choice (then cached).  `tune(m, precision, form, nsteps) -> int` replaces the GPU autotuner
    (tests)."""
    if device_name is None:
        import torch

        device_name = torch.cuda.get_device_name()
    k = key(device_name, m, precision, fused)
    data = load(path)
    if k in data:
        return int(data[k])
    if tune is None:
        from .solver import Solver

        def tune(m_, p_, f_, n_):
            with Solver.from_model(m_, precision=p_, fused=f_) as s:
                return s.autotune(n_)

    best = int(tune(m, precision, fused, nsteps))
    store(k, best, path)
    return best


def split_setting_for(m, precision: int = F.PREC_F32, nsteps: int = 30, path: str | None = None,
                      device_name: str | None = None, tune=None) -> tuple[int, int, int]:
    """The two-kernel step's cached (z-chunk, tile height, L2 prefetch distance) for this workload
    shape, or the autotuner's choice (then cached).  `tune(m, precision, nsteps) -> (kchunk,
    tile_y, l2_prefetch)` replaces the GPU autotuner (tests)."""
    if device_name is None:
        import torch

        device_name = torch.cuda.get_device_name()
    k = key(device_name, m, precision, F.STEP_SPLIT) + "|tile"
    data = load(path)
    v = data.get(k)
    if isinstance(v, list) and len(v) == 3:
        return int(v[0]), int(v[1]), int(v[2])
    if tune is None:
        from .solver import Solver

        def tune(m_, p_, n_):
            with Solver.from_model(m_, precision=p_) as s:
                return s.autotune(n_), s.tile(), s.l2_prefetch()

    kc, ty, pf = (int(x) for x in tune(m, precision, nsteps))
    store(k, [kc, ty, pf], path)
    return kc, ty, pf
