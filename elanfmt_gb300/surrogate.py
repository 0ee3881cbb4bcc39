"""Learned Green's-function surrogate: data from the batched solver, an MLP trained and run by the
project's own CUDA kernels (ewf_mlp_*), the solver as fallback and as the measure of its error.

Network (default, "structured"): (source depth, receiver offset) -> the 10 fundamental traces
of a point moment tensor in a laterally homogeneous medium, which ewf_mlp_combine mixes into the
6 elementary moment tensors x 3 velocity components for the query's azimuth
(mixing_matrices); the other form maps (depth, offset, first and second azimuthal harmonics) to
the 18 traces directly.  4 hidden layers of 512 GELU units, bf16 weights and activations, fp32
accumulation (tcgen05 tensor cores, accumulators in tensor memory), fp32 master weights and Adam.
The forward and backward passes,
the loss gradient, the optimiser and the mixing run in the hand-written kernels of
csrc/ewf_mlp.cu; torch provides the device buffers, the row gathers that form minibatches, and
the sum of the per-block loss partials that is logged.

    python -m elanfmt_gb300.surrogate [--train-runs 256] [--test-runs 64] [--out report.json]
    python -m elanfmt_gb300.surrogate --gemm-bench | --infer-bench | --gemm-once M,N,K
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time

import numpy as np

from . import fields as F
from . import inputs as I
from . import runs
from .solver import Batch, _check, load_library

IN_PAD = 128          # inputs padded to one GEMM tile
NCOMP = 18            # 6 moment tensors x 3 velocity components


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class MLP:
    """bf16 MLP with fp32 master weights; forward/backward/Adam through the ewf_mlp_* kernels."""

    def __init__(self, sizes: list[int], seed: int = 0, fan_in0: int | None = None):
        """sizes[0] is the padded input width (a multiple of 32); fan_in0 the number of input
        columns that carry features (the rest are zero).  Weights: He normal on the effective
        fan-in (1/fan_in for the linear output layer); biases uniform in +-1/sqrt(fan_in), so the
        GELU kinks of the first layer are spread over the input range instead of all sitting at
        the origin (zero biases with zero-padded inputs train about 15x worse on smooth maps)."""
        import torch

        self.torch = torch
        self.lib = load_library()
        self.sizes = sizes
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.W, self.Wb, self.b, self.mW, self.vW, self.mb, self.vb = [], [], [], [], [], [], []
        for l in range(len(sizes) - 1):
            fan_in, fan_out = sizes[l], sizes[l + 1]
            fi = fan_in0 if (l == 0 and fan_in0) else fan_in
            std = math.sqrt(2.0 / fi) if l < len(sizes) - 2 else math.sqrt(1.0 / fi)
            w = torch.randn(fan_out, fan_in, generator=g) * std
            if l == 0 and fan_in0:
                w[:, fan_in0:] = 0.0
            w = w.cuda()
            self.W.append(w)
            self.Wb.append(w.to(torch.bfloat16))
            bnd = 1.0 / math.sqrt(fi)
            self.b.append(((torch.rand(fan_out, generator=g) * 2 - 1) * bnd).cuda())
            for lst in (self.mW, self.vW):
                lst.append(torch.zeros_like(w))
            for lst in (self.mb, self.vb):
                lst.append(torch.zeros(fan_out, device="cuda"))
        self.step_count = 0
        self._ws = {}

    @property
    def nlayers(self) -> int:
        return len(self.sizes) - 1

    def _work(self, M: int) -> dict:
        if M not in self._ws:
            t = self.torch
            s = self.sizes
            w = {"H": [t.empty(M, s[l], dtype=t.bfloat16, device="cuda") for l in range(self.nlayers)],
                 "P": [t.empty(M, s[l + 1], device="cuda") for l in range(self.nlayers - 1)],
                 "Y": t.empty(M, s[-1], device="cuda"),
                 "dY": [t.empty(M, s[l + 1], dtype=t.bfloat16, device="cuda") for l in range(self.nlayers)],
                 "dH": [t.empty(M, s[l], dtype=t.bfloat16, device="cuda") for l in range(self.nlayers)],
                 "dYt": [t.empty(s[l + 1], M, dtype=t.bfloat16, device="cuda") for l in range(self.nlayers)],
                 "Ht": [t.empty(s[l], M, dtype=t.bfloat16, device="cuda") for l in range(self.nlayers)],
                 "Wt": [t.empty(s[l], s[l + 1], dtype=t.bfloat16, device="cuda") for l in range(self.nlayers)],
                 "gW": [t.empty(s[l + 1], s[l], device="cuda") for l in range(self.nlayers)],
                 "gb": [t.empty(s[l + 1], device="cuda") for l in range(self.nlayers)],
                 "part": t.empty(1024, device="cuda")}
            self._ws[M] = w
        return self._ws[M]

    def forward(self, X, Y=None, keep_pre: bool = True) -> "torch.Tensor":
        """X: bf16 [M, sizes[0]] on the GPU; returns the fp32 output [M, sizes[-1]], written into Y
        when given (contiguous rows, e.g. a row slice of the caller's output), else into the
        workspace.  keep_pre=False skips the pre-activations (only the backward pass reads them)."""
        M = X.shape[0]
        w = self._work(M)
        st = _stream()
        w["H"][0].copy_(X)
        Yd = w["Y"] if Y is None else Y
        for l in range(self.nlayers):
            last = l == self.nlayers - 1
            _check(self.lib.ewf_mlp_gemm(_p(w["H"][l]), _p(self.Wb[l]), _p(self.b[l]),
                                         _p(Yd) if last else None, None if last else _p(w["H"][l + 1]),
                                         None if (last or not keep_pre) else _p(w["P"][l]), M, self.sizes[l + 1],
                                         self.sizes[l], 0 if last else 1, st), "ewf_mlp_gemm")
        return Yd

    def loss_grad(self, T) -> "torch.Tensor":
        """MSE against fp32 targets T; dY of the last layer into the workspace; returns the loss."""
        M = T.shape[0]
        w = self._work(M)
        n = w["Y"].numel()
        nb = 1024
        _check(self.lib.ewf_mlp_mse_grad(_p(w["Y"]), _p(T), _p(w["dY"][-1]), n, C.c_float(1.0 / n), _p(w["part"]), nb,
                                         _stream()), "ewf_mlp_mse_grad")
        return w["part"].sum() / n

    def backward(self, M: int) -> None:
        w = self._work(M)
        st = _stream()
        L = self.nlayers
        for l in range(L - 1, -1, -1):
            nout, nin = self.sizes[l + 1], self.sizes[l]
            # dW = dY^T H: A = dY^T [nout, M], B = H^T [nin, M]
            _check(self.lib.ewf_mlp_transpose(_p(w["dY"][l]), _p(w["dYt"][l]), M, nout, st), "transpose")
            _check(self.lib.ewf_mlp_transpose(_p(w["H"][l]), _p(w["Ht"][l]), M, nin, st), "transpose")
            _check(self.lib.ewf_mlp_gemm(_p(w["dYt"][l]), _p(w["Ht"][l]), None, _p(w["gW"][l]), None, None, nout, nin, M,
                                         0, st), "gemm dW")
            _check(self.lib.ewf_mlp_bias_grad(_p(w["dY"][l]), _p(w["gb"][l]), M, nout, st), "bias_grad")
            if l > 0:
                # dH = dY W: A = dY [M, nout], B = W^T [nin, nout]
                _check(self.lib.ewf_mlp_transpose(_p(self.Wb[l]), _p(w["Wt"][l]), nout, nin, st), "transpose")
                _check(self.lib.ewf_mlp_gemm(_p(w["dY"][l]), _p(w["Wt"][l]), None, None, _p(w["dH"][l]), None, M, nin,
                                             nout, 0, st), "gemm dH")
                _check(self.lib.ewf_mlp_gelu_grad(_p(w["dH"][l]), _p(w["P"][l - 1]), _p(w["dY"][l - 1]), w["dH"][l].numel(),
                                                  st), "gelu_grad")

    def adam(self, M: int, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8, wd: float = 0.0) -> None:
        w = self._work(M)
        self.step_count += 1
        st = _stream()
        for l in range(self.nlayers):
            _check(self.lib.ewf_mlp_adam(_p(self.W[l]), _p(self.mW[l]), _p(self.vW[l]), _p(w["gW"][l]), _p(self.Wb[l]),
                                         self.W[l].numel(), C.c_float(lr), C.c_float(b1), C.c_float(b2), C.c_float(eps),
                                         self.step_count, C.c_float(wd), st), "adam W")
            _check(self.lib.ewf_mlp_adam(_p(self.b[l]), _p(self.mb[l]), _p(self.vb[l]), _p(w["gb"][l]), None,
                                         self.b[l].numel(), C.c_float(lr), C.c_float(b1), C.c_float(b2), C.c_float(eps),
                                         self.step_count, C.c_float(0.0), st), "adam b")

    def check_status(self) -> None:
        """Raises if a GEMM launch since the last check gave up on a bounded wait (its outputs, and
        everything computed from them, are invalid).  Synchronises the device."""
        _check(self.lib.ewf_mlp_status(), "ewf_mlp_status")

    def train(self, X, T, steps: int, batch: int = 256, lr: float = 1e-3, seed: int = 0, log_every: int = 0) -> list:
        """X: bf16 [n, sizes[0]], T: fp32 [n, sizes[-1]] on the GPU.  Cosine learning-rate decay.
        The GEMMs' status is checked at every logged step and at the end."""
        torch = self.torch
        n = X.shape[0]
        g = torch.Generator(device="cuda").manual_seed(seed)
        losses = []
        for s in range(steps):
            idx = torch.randint(0, n, (batch,), device="cuda", generator=g)
            self.forward(X.index_select(0, idx))
            loss = self.loss_grad(T.index_select(0, idx))
            self.backward(batch)
            self.adam(batch, lr * 0.5 * (1 + math.cos(math.pi * s / steps)))
            if log_every and (s % log_every == 0 or s == steps - 1):
                self.check_status()
                losses.append((s, float(loss)))
        self.check_status()
        return losses

    def predict(self, X, batch: int = 8192):
        """Inference of X [n, sizes[0]] in batches of `batch` rows: full batches write their rows of
        the output directly; a ragged last batch is padded to 128 rows and copied."""
        torch = self.torch
        n = X.shape[0]
        out = torch.empty(n, self.sizes[-1], device="cuda")
        for a in range(0, n, batch):
            xb = X[a:a + batch]
            m = xb.shape[0]
            if m % 128 == 0:
                self.forward(xb, out[a:a + m], keep_pre=False)
                continue
            pad = torch.zeros(128 - m % 128, X.shape[1], dtype=X.dtype, device="cuda")
            y = self.forward(torch.cat([xb, pad]), keep_pre=False)
            out[a:a + m] = y[:m]
        self.check_status()
        return out


# ---------------------------------------------------------------------------------------------
# data from the solver
# ---------------------------------------------------------------------------------------------

def layered_iso(n: int = 192, dx: float = 120.0, nt: int = 1024, nlayers: int = 8, seed: int = 11, f0: float = 0.5,
                lpml: int = 15):
    """Layered isotropic model on the orthorhombic scheme (C11=C22=C33, C12=C13=C23, C44=C55=C66
    per layer), PML on x, y and the bottom, free surface on top."""
    rng = np.random.default_rng(seed)
    vp = np.sort(rng.uniform(3000, 6500, nlayers))
    vs = vp / rng.uniform(1.65, 1.85, nlayers)
    rho = np.sort(rng.uniform(2200, 2900, nlayers))
    li = I.layer_index(n, nlayers)
    lam = rho * (vp ** 2 - 2 * vs ** 2)
    mu = rho * vs ** 2
    vmax = float(vp.max())
    dt = 0.5 * dx / (vmax * math.sqrt(3.0))
    m = I.Model(nx=n, ny=n, nz=n, nt=nt, dx=float(np.float32(dx)), dy=float(np.float32(dx)), dz=float(np.float32(dx)),
                dt=float(np.float32(dt)), model=F.MODEL_ORTHO, damping=F.DAMP_SEPARABLE, src_order=F.SRC_AFTER_BC1,
                name=f"layered_iso{n}")
    full = lambda v: np.broadcast_to(v[li][:, None, None], (n, n, n))  # noqa: E731
    c11 = (lam + 2 * mu)
    for fid in (F.M_C11, F.M_C22, F.M_C33):
        m.materials[fid] = np.ascontiguousarray(full(c11).astype(np.float32))
    for fid in (F.M_C12, F.M_C13, F.M_C23):
        m.materials[fid] = np.ascontiguousarray(full(lam).astype(np.float32))
    m.materials[F.M_C44YZ] = I.harmonic_edges(full(mu), "yz")
    m.materials[F.M_C55XZ] = I.harmonic_edges(full(mu), "xz")
    m.materials[F.M_C66XY] = I.harmonic_edges(full(mu), "xy")
    b = full(1.0 / rho)
    m.materials[F.M_BX] = I.staggered_buoyancy(b, "x")
    m.materials[F.M_BY] = I.staggered_buoyancy(b, "y")
    m.materials[F.M_BZ] = I.staggered_buoyancy(b, "z")
    m.damping_arrays[F.D_WX] = I.pml_factors(n, lpml, m.dt)
    m.damping_arrays[F.D_WY] = I.pml_factors(n, lpml, m.dt)
    m.damping_arrays[F.D_WZ] = I.pml_factors(n, lpml, m.dt, sides="high")
    m.stf = I.ricker_stf(nt, m.dt, f0, t0=1.0 / f0, scale=1.0 / (m.dx * m.dy * m.dz))
    m.meta = dict(vp=vp.tolist(), vs=vs.tolist(), rho=rho.tolist(), f0=f0, lpml=lpml)
    return m


def surface_receivers(n: int, lpml: int, step: int) -> np.ndarray:
    coords = list(range(lpml + 1, n - lpml - 1, step))
    return np.array([(i, j) for j in coords for i in coords], np.int32)


# each receiver records both staggered samples of each velocity component around the centre of
# its cell (Vx[i'] sits at x = i' - 1/2, Vy[j'] at y = j' - 1/2, Vz[k'] at z = k' - 1/2); their mean
# is the component at the cell centre, so that all three components share one position
_REC_PAIRS = ((F.F_VX, 0, 0, 0), (F.F_VX, 1, 0, 0), (F.F_VY, 0, 0, 0), (F.F_VY, 0, 1, 0), (F.F_VZ, 0, 0, 0),
              (F.F_VZ, 0, 0, 1))


def generate(m, sources: np.ndarray, picks: list, rec_xy: np.ndarray, runs_per_batch: int = 10, log=None,
             decimate: int = 1):
    """Runs the 6 elementary moment tensors for every source cell (xs, ys, zs) with the batched
    solver (one problem whose right-hand sides are 6 per source, each a co-located point source)
    and returns, per source, the velocity traces [npick, 18, nt / decimate] (float32; every
    `decimate`-th time step) at the centres of its picked receiver cells (indices into rec_xy,
    depth cell 1), plus the device seconds per source."""
    out = []
    secs = 0.0
    for a in range(0, len(sources), runs_per_batch):
        chunk = list(range(a, min(a + runs_per_batch, len(sources))))
        union = sorted(set(int(r) for s in chunk for r in picks[s]))
        pos = {r: q for q, r in enumerate(union)}
        rec = np.array([(rec_xy[r][0] + di, rec_xy[r][1] + dj, 1 + dk, c) for r in union for c, di, dj, dk in _REC_PAIRS],
                       np.int32)
        mm = I.Model(**{k: getattr(m, k) for k in ("nx", "ny", "nz", "nt", "dx", "dy", "dz", "dt", "model", "damping",
                                                    "src_order")})
        mm.materials, mm.damping_arrays, mm.stf, mm.receivers = m.materials, m.damping_arrays, m.stf, rec
        rl = []
        for s in chunk:
            xs, ys, zs = (int(v) for v in sources[s])
            for q in range(6):
                mt = np.zeros(6)
                mt[q] = 1.0
                rl.append(F.mt_point_entries(mt, xs, ys, zs))
        with Batch([(mm, rl)]) as b:
            secs += b.run(m.nt) * 1e-3
            for u, s in enumerate(chunk):
                sel = np.array([pos[int(r)] for r in picks[s]])
                tr = np.empty((len(sel), NCOMP, len(range(0, m.nt, decimate))), np.float32)
                for q in range(6):
                    t = b.seismograms(0, 6 * u + q).reshape(len(union), 3, 2, m.nt).mean(axis=2)
                    tr[:, 3 * q:3 * q + 3, :] = t[sel][..., ::decimate]
                out.append(tr)
        if log:
            log(f"generated {chunk[-1] + 1}/{len(sources)} sources")
    return out, secs / len(sources)


def geometry(m, src: np.ndarray, rec_xy: np.ndarray) -> np.ndarray:
    """Per (source, receiver): (depth, offset, azimuth, distance, source x, source y) in metres /
    radians.  The model is laterally homogeneous, so the first three determine the Green's
    functions up to the PML's influence (which the source position carries)."""
    xs, ys, zs = (src[:, None, 0] * m.dx, src[:, None, 1] * m.dy, src[:, None, 2] * m.dz)
    dxr = rec_xy[None, :, 0] * m.dx - xs
    dyr = rec_xy[None, :, 1] * m.dy - ys
    off = np.hypot(dxr, dyr)
    az = np.arctan2(dyr, dxr)
    depth = np.broadcast_to(zs, off.shape)
    return np.stack([depth, off, az, np.hypot(off, depth), np.broadcast_to(xs, off.shape),
                     np.broadcast_to(ys, off.shape)], axis=-1)


def features(geo: np.ndarray, structured: bool, az4: bool = False, full: bool = False) -> np.ndarray:
    """Network inputs.  structured: (depth, offset) -- the network predicts the fundamental traces,
    which do not depend on azimuth in a laterally homogeneous medium; az4 adds cos 4az, sin 4az,
    the lowest harmonic of a cubic grid's direction-dependent dispersion.  Otherwise (depth,
    offset, cos az, sin az, cos 2az, sin 2az): the radiation patterns of the elementary moment
    tensors are combinations of the first and second azimuthal harmonics; `full` adds the source's
    x and y (the five inputs source x, y, depth, receiver offset, azimuth, with no symmetry
    assumed)."""
    depth, off, az = geo[..., 0], geo[..., 1], geo[..., 2]
    if structured:
        cols = [depth, off] + ([np.cos(4 * az), np.sin(4 * az)] if az4 else [])
        return np.stack(cols, axis=-1).astype(np.float32)
    cols = [depth, off, np.cos(az), np.sin(az), np.cos(2 * az), np.sin(2 * az)]
    if full:
        cols = [geo[..., 4], geo[..., 5]] + cols
    return np.stack(cols, axis=-1).astype(np.float32)


NFUND = 10            # fundamental traces of a point moment tensor in a laterally homogeneous medium
_MT_PAIRS = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))   # xx, yy, zz, xy, xz, yz


def mixing_matrices(az: np.ndarray) -> np.ndarray:
    """R [n, 18, 10] with traces[3q + c] = R[3q + c] . fundamentals, for the 6 elementary moment
    tensors q and the x, y, z velocity components c of a receiver at azimuth az from the source.

    In the frame turned to the receiver (x' radial, y' transverse, z), mirror symmetry about the
    x'z plane leaves the vertical and radial motion depending on M'xx, M'yy, M'zz, M'xz only and
    the transverse motion on M'xy, M'yz only, each through a trace that depends on depth and
    offset but not azimuth: fundamentals 0-3 (vertical), 4-7 (radial), 8-9 (transverse), with
    M' = Q M Q^T, Q = [r; t; z], r = (cos az, sin az, 0), t = (-sin az, cos az, 0)."""
    az = np.asarray(az, np.float64)
    c, s = np.cos(az), np.sin(az)
    n = len(az)
    Q = np.zeros((n, 3, 3))
    Q[:, 0, 0], Q[:, 0, 1], Q[:, 1, 0], Q[:, 1, 1], Q[:, 2, 2] = c, s, -s, c, 1.0
    R = np.zeros((n, NCOMP, NFUND))
    for q, (i, j) in enumerate(_MT_PAIRS):
        E = np.zeros((3, 3))
        E[i, j] = E[j, i] = 1.0
        Mp = Q @ E @ Q.transpose(0, 2, 1)
        rz = np.stack([Mp[:, 0, 0], Mp[:, 1, 1], Mp[:, 2, 2], Mp[:, 0, 2]], axis=-1)
        tt = np.stack([Mp[:, 0, 1], Mp[:, 1, 2]], axis=-1)
        R[:, 3 * q + 0, 4:8] = c[:, None] * rz
        R[:, 3 * q + 0, 8:10] = -s[:, None] * tt
        R[:, 3 * q + 1, 4:8] = s[:, None] * rz
        R[:, 3 * q + 1, 8:10] = c[:, None] * tt
        R[:, 3 * q + 2, 0:4] = rz
    return R.astype(np.float32)


def fundamentals(Y: np.ndarray, R: np.ndarray) -> np.ndarray:
    """Least-squares fundamental traces [n, 10, nt] of each GF set Y [n, 18*nt] (18 equations, 10
    unknowns per time sample); the residual measures how far the solver's traces are from the
    symmetry (grid anisotropy, staggered receiver positions, PML)."""
    n = len(Y)
    P = np.linalg.pinv(R.astype(np.float64)).astype(np.float32)     # [n, 10, 18]
    out = np.empty((n, NFUND, Y.shape[1] // NCOMP), np.float32)
    for a in range(0, n, 1024):
        out[a:a + 1024] = P[a:a + 1024] @ Y[a:a + 1024].reshape(-1, NCOMP, Y.shape[1] // NCOMP)
    return out


def rel_l2(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Relative L2 error per row (GF set) of a against b."""
    a = a.reshape(len(a), -1).astype(np.float64)
    b = b.reshape(len(b), -1).astype(np.float64)
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def make_dataset(train_runs: int = 256, test_runs: int = 64, n: int = 192, nt: int = 1280, per_run: int = 64,
                 seed: int = 7, max_offset: float = 12000.0, log=print, f0: float = 0.5, decimate: int = 1,
                 dx: float = 120.0, pml_m: float = 1800.0) -> dict | None:
    """Runs the solver for train_runs + test_runs random source cells (depth 2-8 km, scaled to the
    grid) for nt time steps and keeps, per source, `per_run` receivers with offsets in 1 km ..
    max_offset, every `decimate`-th sample.  Under torch.distributed the sources are shared out
    over the ranks (elanfmt_gb300.runs) and only rank 0 gets the dataset (None elsewhere)."""
    # geometry in metres (the cell counts below are those of dx = 120 m): a pml_m (1.8 km) PML,
    # receivers every 360 m, sources from 1.2 km inside the PML over 4 km
    m = layered_iso(n=n, nt=nt, f0=f0, dx=dx, lpml=int(round(pml_m / dx)))
    lpml = m.meta["lpml"]
    rec_xy = surface_receivers(n, lpml, max(1, int(round(360.0 / dx))))
    rng = np.random.default_rng(seed)
    nrun = train_runs + test_runs
    zlo = int(round(2000 / m.dz))
    zhi = min(int(round(8000 / m.dz)), n - lpml - 4)
    x0 = lpml + int(round(1200.0 / dx))
    span = max(4, min(int(4000 / m.dx), n - lpml - x0 - int(round(1200.0 / dx))))
    src = np.stack([rng.integers(x0, x0 + span, nrun), rng.integers(x0, x0 + span, nrun),
                    rng.integers(zlo, zhi + 1, nrun)], axis=1).astype(np.int32)
    geo = geometry(m, src, rec_xy)                         # [nrun, nrec, 4]
    picks = []
    for s in range(nrun):
        ok = np.nonzero((geo[s, :, 1] >= 1000) & (geo[s, :, 1] <= max_offset))[0]
        picks.append(np.sort(rng.choice(ok, size=min(per_run, len(ok)), replace=False)))
    # independent solves: under torch.distributed every rank generates its share of the sources
    # on its GPU and rank 0 gathers the traces (host side) and goes on alone
    dist = _dist()
    rank, world = (dist.get_rank(), dist.get_world_size()) if dist else (0, 1)
    mine = list(runs.shard(nrun, rank, world))
    t0 = time.perf_counter()
    local, fdtd_s_per_src = generate(m, src[mine], [picks[s] for s in mine], rec_xy, log=log, decimate=decimate)
    got = runs.gather(dict(zip(mine, local)), dist)
    if got is None:
        return None
    traces = [got[s] for s in range(nrun)]
    log(f"data: {nrun} sources on {world} GPU(s) in {time.perf_counter() - t0:.1f} s "
        f"({fdtd_s_per_src:.3f} device s per source, 6 RHS)")
    samples_src = np.concatenate([[s] * len(picks[s]) for s in range(nrun)]).astype(np.int64)
    samples_rec = np.concatenate(picks)
    return dict(m=m, rec_xy=rec_xy, src=src, train_runs=train_runs, test_runs=test_runs, per_run=per_run,
                decimate=decimate, max_offset=max_offset,
                samples_src=samples_src, geo=geo[samples_src, samples_rec],
                Y=np.concatenate([t.reshape(len(t), -1) for t in traces]), fdtd_s_per_src=fdtd_s_per_src)


def fourier_features(Xs: np.ndarray, sigma: float, width: int, seed: int = 0) -> np.ndarray:
    """[Xs, sin(2 pi Xs B^T), cos(2 pi Xs B^T)] with B ~ N(0, sigma^2) (random Fourier features,
    Tancik et al. 2020: an MLP fed with them fits oscillatory functions of its inputs far better),
    `width` columns in all; sigma = 0 returns Xs."""
    if sigma <= 0:
        return Xs
    nf = (width - Xs.shape[1]) // 2
    B = np.random.default_rng(seed).normal(0.0, sigma, size=(nf, Xs.shape[1]))
    proj = 2 * np.pi * Xs.astype(np.float64) @ B.T
    return np.concatenate([Xs, np.sin(proj), np.cos(proj)], axis=1).astype(np.float32)


def fit_and_evaluate(ds: dict, steps: int = 6000, seed: int = 7, hidden: int = 512, layers: int = 4,
                     lr: float = 1e-3, spreading: bool = True, structured: bool = True, fourier: float = 0.0,
                     az4: bool = False, full: bool = False, log=print) -> dict:
    """Trains the MLP on the training sources of a dataset and scores it on the held-out ones
    against the solver's traces; also scores the nearest-neighbour method (no network) and the
    fallback policy.  structured: the network maps (depth, offset) to the 10 fundamental traces
    and ewf_mlp_combine mixes them into the 18 traces of each receiver's azimuth; otherwise it maps
    (depth, offset, azimuth harmonics) to the 18 traces directly."""
    import torch

    m, Y, geo, samples_src = ds["m"], ds["Y"], ds["geo"], ds["samples_src"]
    lib = load_library()
    nt = Y.shape[1] // NCOMP
    train_runs = ds["train_runs"]
    is_train = samples_src < train_runs
    val_src = samples_src < max(1, train_runs // 10)      # a tenth of the training sources validates
    fit = is_train & ~val_src
    # GF sets whose recorded energy is negligible (nothing arrived in the window) carry no
    # meaningful relative error; they are left out of the error statistics and counted
    energy = np.linalg.norm(Y.astype(np.float64), axis=1)
    live = energy > 1e-3 * np.median(energy)
    test = ~is_train & live
    val_src = val_src & live
    if full:
        structured = False
    X = features(geo, structured, az4, full)
    mu, sd = X[fit].mean(axis=0), X[fit].std(axis=0) + 1e-6
    Xs = (X - mu) / sd
    # geometric spreading: targets scaled by distance, so that near and far receivers weigh alike
    # in the loss as they do in the per-set relative error
    amp = (geo[:, 3] / np.median(geo[:, 3])).astype(np.float32) if spreading else np.ones(len(X), np.float32)
    R = mixing_matrices(geo[:, 2])
    if structured:
        Gf = fundamentals(Y, R)
        sym_err = rel_l2(np.einsum("nof,nft->not", R[test], Gf[test]), Y[test])
        T = Gf.reshape(len(Gf), -1) * amp[:, None]
        del Gf
    else:
        sym_err = None
        T = Y * amp[:, None]
    nout = T.shape[1]
    fit_rows = np.nonzero(fit)[0]
    scale = float(np.sqrt(np.mean(T[fit_rows] ** 2)))
    Xf_in = fourier_features(Xs, fourier, IN_PAD, seed)
    Xp = np.zeros((len(X), IN_PAD), np.float32)
    Xp[:, :Xf_in.shape[1]] = Xf_in
    Xg = torch.from_numpy(Xp).cuda().to(torch.bfloat16)
    Tg = torch.from_numpy(T / scale).cuda()
    fit_idx = torch.from_numpy(fit_rows).cuda()
    net = MLP([IN_PAD] + [hidden] * layers + [nout], seed=seed, fan_in0=Xf_in.shape[1])
    t0 = time.perf_counter()
    losses = net.train(Xg.index_select(0, fit_idx), Tg.index_select(0, fit_idx), steps=steps, batch=256, lr=lr,
                       log_every=max(1, steps // 10))
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    log(f"trained {steps} steps in {train_s:.1f} s; loss {losses[0][1]:.4g} -> {losses[-1][1]:.4g}")
    Rg = torch.from_numpy(R).cuda()

    def infer(idx):
        """GF sets of the samples idx (device index tensor), in the network's scaled units."""
        y = net.predict(Xg.index_select(0, idx))
        if not structured:
            return y
        out = torch.empty(len(idx), NCOMP * nt, device="cuda")
        rq = Rg.index_select(0, idx)
        for a in range(0, len(idx), 32768):
            b = min(a + 32768, len(idx))
            _check(lib.ewf_mlp_combine(_p(rq[a:b]), _p(y[a:b]), _p(out[a:b]), b - a, NCOMP, NFUND, nt, _stream()),
                   "ewf_mlp_combine")
        return out

    def predict(mask):
        idx = torch.from_numpy(np.nonzero(mask)[0]).cuda()
        return infer(idx).cpu().numpy() * scale / amp[mask][:, None]

    err_test = rel_l2(predict(test), Y[test])
    err_val = rel_l2(predict(val_src), Y[val_src])
    # error predictor: the mean error of the 5 nearest validation samples in feature space
    Xv, Xt = Xs[val_src], Xs[test]
    d2 = ((Xt[:, None, :] - Xv[None, :, :]) ** 2).sum(-1)
    nn5 = np.argsort(d2, axis=1)[:, :5]
    pred_err = err_val[nn5].mean(axis=1)
    accept = pred_err <= 1e-3
    # the method without the network: the nearest training sample in the same feature space, with
    # the same spreading correction (and, structured, its fundamentals mixed for the query's azimuth)
    Xf = Xs[fit]
    nn1 = fit_rows[np.concatenate([np.argmin(((Xt[a:a + 256, None, :] - Xf[None, :, :]) ** 2).sum(-1), axis=1)
                                   for a in range(0, len(Xt), 256)])]
    amp_t = amp[test][:, None]
    if structured:
        near = np.einsum("nof,nft->not", R[test], T[nn1].reshape(-1, NFUND, nt)).reshape(len(nn1), -1)
    else:
        near = T[nn1]
    err_nn = rel_l2(near / amp_t, Y[test])
    # throughput: surrogate inference of every test query (CUDA events) vs FDTD per source
    idx = torch.from_numpy(np.nonzero(test)[0]).cuda()
    infer(idx)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    reps = 20
    for _ in range(reps):
        infer(idx)
    e1.record()
    torch.cuda.synchronize()
    surr_s = e0.elapsed_time(e1) * 1e-3 / reps
    nq = int(test.sum())
    fdtd_s_per_src = ds["fdtd_s_per_src"]
    per_run = ds["per_run"]
    surr_rate = nq / surr_s
    fdtd_rate_recorded = len(ds["rec_xy"]) / fdtd_s_per_src   # every recorded receiver of a run
    fdtd_rate_queried = per_run / fdtd_s_per_src              # the receivers actually queried per run
    # with fallback: accepted queries from the network, the rest from one FDTD run per source
    fb_sources = len(np.unique(samples_src[test][~accept]))
    eff_s = surr_s + fb_sources * fdtd_s_per_src
    eff_err = np.where(accept, err_test, 0.0)
    n = m.nx

    def stats(e):
        return {"median": float(np.median(e)), "p90": float(np.percentile(e, 90)), "min": float(e.min()),
                "max": float(e.max()), "frac_le_1e-3": float((e <= 1e-3).mean()),
                "frac_le_1e-2": float((e <= 1e-2).mean()), "frac_le_1e-1": float((e <= 1e-1).mean())}

    return {
        "model": f"layered isotropic {n}^3, dx {m.dx:.0f} m, 8 layers, {m.nt} steps recorded every "
                 f"{ds.get('decimate', 1)} -> {nt} samples, Ricker {m.meta['f0']} Hz, offsets 1 km - "
                 f"{ds.get('max_offset', 12000.0) / 1000:.0f} km",
        "train_sources": train_runs, "test_sources": ds["test_runs"], "receivers_recorded": int(len(ds["rec_xy"])),
        "queries_per_source": per_run, "train_samples": int(fit.sum()), "val_samples": int(val_src.sum()),
        "test_samples": nq, "test_samples_without_energy": int((~is_train & ~live).sum()),
        "network": f"MLP {X.shape[1]}(->{IN_PAD} pad) -> {layers}x{hidden} GELU -> {nout}, bf16 weights, "
                   "fp32 accumulate",
        "structured": structured,
        "fourier_sigma": fourier, "az4": az4,
        "features": ("depth, offset -> 10 fundamental traces, mixed per azimuth" if structured else
                     ("source x, y, " if full else "") + "depth, offset, cos/sin az, cos/sin 2az -> 18 traces")
                    + " (standardised)" +
                    ("; targets x distance" if spreading else ""),
        "symmetry_floor_rel_l2": stats(sym_err) if structured else None,
        "train_steps": steps, "train_seconds": round(train_s, 2), "loss_first_last": [losses[0][1], losses[-1][1]],
        "surrogate_rel_l2": stats(err_test),
        "nearest_neighbour_rel_l2": stats(err_nn),
        "network_gain_median": float(np.median(err_nn) / max(np.median(err_test), 1e-300)),
        "accepted_by_error_predictor": float(accept.mean()),
        "accepted_true_error_max": float(err_test[accept].max()) if accept.any() else None,
        "gf_sets_per_s": {"surrogate": surr_rate, "fdtd_all_recorded_receivers": fdtd_rate_recorded,
                          "fdtd_queried_receivers": fdtd_rate_queried,
                          "surrogate_over_fdtd_all": surr_rate / fdtd_rate_recorded,
                          "with_fallback": nq / eff_s, "with_fallback_over_fdtd_queried": (nq / eff_s) / fdtd_rate_queried},
        "fallback_sources": int(fb_sources), "effective_max_rel_l2_served": float(eff_err.max()),
        "fdtd_device_seconds_per_source": fdtd_s_per_src,
    }


def symmetry_floor(cases=((0.5, 120.0), (0.5, 60.0)), sources: int = 16, n120: int = 192, per_run: int = 64,
                   max_offset: float = 12000.0, seed: int = 9, steps_at_half_hz: int = 1280, log=print) -> list:
    """How far the solver's own traces are from the lateral symmetry that the structured surrogate
    assumes, against grid resolution and absorbing boundary: for each (Ricker peak frequency f0,
    cell size dx[, absorbing layer thickness in metres, default 1800, and cells of 120 m added on
    every side]), the same physical model (n120 cells of 120 m, so n120 * 120 / dx cells), `sources` random source
    cells, the 18 traces of `per_run` receivers (offset 1 km .. max_offset), and the relative L2
    residual of their best fit by 10 azimuth-independent fundamental traces (`fundamentals`),
    overall and by offset.  The window is steps_at_half_hz steps of the 120 m grid at 0.5 Hz,
    longer as 1/f0 and finer grids take more steps, so every case sees the same arrivals.  Points
    per wavelength are given at f0 and at 2.5 f0 (the Ricker spectrum's upper edge) for the
    slowest S velocity."""
    out = []
    for case in cases:
        f0, dx = case[0], case[1]
        pml_m = case[2] if len(case) > 2 else 1800.0
        n = int(round((n120 + 2 * round((pml_m - 1800.0) / 120.0)) * 120.0 / dx))
        nt = int(round(steps_at_half_hz * (0.5 / f0) * (120.0 / dx)))
        ds = make_dataset(train_runs=sources, test_runs=0, n=n, nt=nt, per_run=per_run, seed=seed,
                          max_offset=max_offset, log=log, f0=f0, dx=dx, pml_m=pml_m)
        if ds is None:
            return []
        m, Y, geo = ds["m"], ds["Y"], ds["geo"]
        energy = np.linalg.norm(Y.astype(np.float64), axis=1)
        live = energy > 1e-3 * np.median(energy)
        R = mixing_matrices(geo[:, 2])
        G = fundamentals(Y[live], R[live])
        err = rel_l2(np.einsum("nof,nft->not", R[live], G), Y[live])
        off = geo[live, 1]
        vs_min = float(min(m.meta["vs"]))
        bins = {}
        for lo, hi in ((1000, 4000), (4000, 8000), (8000, 12000), (12000, 20000)):
            sel = (off >= lo) & (off < hi)
            if sel.any():
                bins[f"{lo // 1000}-{hi // 1000} km"] = {"median": float(np.median(err[sel])), "n": int(sel.sum())}
        out.append({"f0_hz": f0, "dx_m": float(m.dx), "pml_m": pml_m, "n": n, "steps": nt,
                    "points_per_s_wavelength_at_f0": vs_min / f0 / m.dx,
                    "points_per_s_wavelength_at_2.5f0": vs_min / (2.5 * f0) / m.dx,
                    "gf_sets": int(live.sum()), "median": float(np.median(err)),
                    "p90": float(np.percentile(err, 90)), "by_offset": bins})
        log(f"f0 {f0} dx {dx} pml {pml_m}: floor median {out[-1]['median']:.4f}, p90 {out[-1]['p90']:.4f}")
    return out


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def study(train_runs: int = 256, test_runs: int = 64, n: int = 192, nt: int = 1280, per_run: int = 64,
          steps: int = 6000, seed: int = 7, max_offset: float = 12000.0, log=print, decimate: int = 1,
          forms=("structured",), **fit_kw) -> dict | None:
    """The whole study (one dataset, one fit per network form: "structured", "harmonics" or
    "full"); None on ranks other than 0 of a multi-GPU run."""
    ds = make_dataset(train_runs, test_runs, n, nt, per_run, seed, max_offset, log, decimate=decimate)
    if ds is None:
        return None
    res = {}
    for form in forms:
        kw = dict(fit_kw, structured=form == "structured", full=form == "full")
        res[form] = fit_and_evaluate(ds, steps=steps, seed=seed, log=log, **kw)
    return res[forms[0]] if len(forms) == 1 else res


def gemm_benchmark(shapes=((4096, 12800, 512), (4096, 512, 512), (256, 12800, 512), (12800, 512, 256),
                            (8192, 8192, 8192)), reps: int = 20) -> list:
    """TFLOP/s of ewf_mlp_gemm (C = A.B^T, bf16 in, fp32 out) against cuBLAS (torch.matmul, bf16 in,
    fp32 accumulate) on the network's shapes (inference output layer, hidden layer, one training
    batch, a weight gradient) and one large square problem; CUDA events, warm."""
    import torch

    lib = load_library()
    out = []
    g = torch.Generator(device="cpu").manual_seed(0)
    for M, N, K in shapes:
        A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
        B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
        C = torch.empty(M, N, device="cuda")
        st = _stream()

        def ours():
            _check(lib.ewf_mlp_gemm(_p(A), _p(B), None, _p(C), None, None, M, N, K, 0, st), "ewf_mlp_gemm")

        def cublas():
            torch.matmul(A, B.T, out=Cb)

        Cb = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
        res = {"M": M, "N": N, "K": K}
        for name, fn in (("ewf_mlp_gemm", ours), ("cublas_bf16", cublas)):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            res[name] = {"ms": round(ms, 4), "tflops": round(2.0 * M * N * K / (ms * 1e-3) / 1e12, 1)}
        out.append(res)
    return out


def infer_benchmark(nq: int = 4096, nt: int = 1280, hidden: int = 512, layers: int = 4, reps: int = 20) -> dict:
    """GF sets/s of surrogate inference at the study's network size, with random weights and
    inputs: the forward pass (ewf_mlp_gemm, batches of 1024 queries as in MLP.predict) and the
    azimuthal mixing (ewf_mlp_combine) of nq queries, timed with CUDA events as in study()."""
    import torch

    lib = load_library()
    net = MLP([IN_PAD] + [hidden] * layers + [NFUND * nt], seed=1, fan_in0=4)
    g = torch.Generator(device="cpu").manual_seed(2)
    X = torch.randn(nq, IN_PAD, generator=g).to(torch.bfloat16).cuda()
    R = torch.randn(nq, NCOMP, NFUND, generator=g).cuda()
    out = torch.empty(nq, NCOMP * nt, device="cuda")

    def infer():
        y = net.predict(X)
        for a in range(0, nq, 32768):
            b = min(a + 32768, nq)
            _check(lib.ewf_mlp_combine(_p(R[a:b]), _p(y[a:b]), _p(out[a:b]), b - a, NCOMP, NFUND, nt, _stream()),
                   "ewf_mlp_combine")

    infer()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        infer()
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) * 1e-3 / reps
    _check(lib.ewf_mlp_status(), "ewf_mlp_status")
    return {"queries": nq, "seconds": sec, "gf_sets_per_s": nq / sec,
            "network": f"{IN_PAD} -> {layers}x{hidden} GELU -> {NFUND * nt} (bf16, fp32 accumulate), + mixing to "
                       f"{NCOMP} x {nt}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gemm-bench", action="store_true", help="only time ewf_mlp_gemm against cuBLAS")
    ap.add_argument("--infer-bench", action="store_true", help="only time inference at the study's network size")
    ap.add_argument("--gemm-once", default="", help="M,N,K: three ewf_mlp_gemm launches of one shape (profiling)")
    ap.add_argument("--train-runs", type=int, default=256)
    ap.add_argument("--test-runs", type=int, default=64)
    ap.add_argument("--n", type=int, default=192)
    ap.add_argument("--nt", type=int, default=1280)
    ap.add_argument("--per-run", type=int, default=64)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--max-offset", type=float, default=12000.0)
    ap.add_argument("--decimate", type=int, default=1, help="keep every d-th time step of the traces")
    ap.add_argument("--forms", default="structured", help="comma list of structured, harmonics, full")
    ap.add_argument("--floor", action="store_true", help="only the symmetry-floor study against f0")
    ap.add_argument("--floor-cases", default="", help="f0:dx[:pml_m],... (default 0.5:120,0.25:120,0.5:60)")
    ap.add_argument("--out", default="")
    a = ap.parse_args()
    import os

    import torch

    if a.gemm_once:
        import ctypes as C

        M, N, K = (int(v) for v in a.gemm_once.split(","))
        lib = load_library()
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
        Cf = torch.empty(M, N, device="cuda")
        for _ in range(3):
            _check(lib.ewf_mlp_gemm(_p(A), _p(B), None, _p(Cf), None, None, M, N, K, 0, None), "ewf_mlp_gemm")
        torch.cuda.synchronize()
        _check(lib.ewf_mlp_status(), "ewf_mlp_status")
        print("ok", M, N, K)
        return
    if a.infer_bench:
        res = infer_benchmark(nt=a.nt)
        print(json.dumps(res, indent=1))
        return
    if a.gemm_bench:
        res = gemm_benchmark()
        print(json.dumps(res, indent=1))
        if a.out:
            with open(a.out, "w") as fh:
                json.dump(res, fh, indent=1)
        return

    if int(os.environ.get("WORLD_SIZE", "1")) > 1:  # torchrun: one rank per GPU, data generation sharded
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    if a.floor:
        cases = ((0.5, 120.0), (0.25, 120.0), (0.5, 60.0)) if not a.floor_cases else \
            tuple(tuple(float(v) for v in c.split(":")) for c in a.floor_cases.split(","))
        res = symmetry_floor(cases=cases, n120=a.n, per_run=a.per_run, max_offset=a.max_offset)
    else:
        res = study(a.train_runs, a.test_runs, a.n, a.nt, per_run=a.per_run, steps=a.steps, max_offset=a.max_offset,
                    decimate=a.decimate, forms=tuple(a.forms.split(",")))
    if res is None:
        return
    print(json.dumps(res, indent=1))
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(res, fh, indent=1)


if __name__ == "__main__":
    main()
