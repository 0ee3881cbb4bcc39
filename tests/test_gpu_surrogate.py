"""Kernels of the learned surrogate (ewf_mlp_*) against torch references and the FP64 oracle."""
import ctypes as C

import numpy as np
import pytest

from elanfmt_gb300.solver import load_library
from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr())


def test_gemm_matches_fp32_reference(cuda_device):
    import torch

    lib = load_library()
    g = torch.Generator(device="cpu").manual_seed(0)
    for M, N, K in ((128, 128, 32), (256, 384, 96), (384, 256, 512)):
        A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
        B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
        bias = torch.randn(N, generator=g).cuda()
        Cf = torch.empty(M, N, device="cuda")
        Cb = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
        pre = torch.empty(M, N, device="cuda")
        assert lib.ewf_mlp_gemm(_p(A), _p(B), _p(bias), _p(Cf), _p(Cb), _p(pre), M, N, K, 1, None) == 0
        torch.cuda.synchronize()
        ref_pre = A.double() @ B.double().T + bias.double()
        assert (pre.double() - ref_pre).norm() / ref_pre.norm() < 1e-6
        ref = torch.nn.functional.gelu(ref_pre)
        assert (Cf.double() - ref).norm() / ref.norm() < 1e-6
        assert (Cb.double() - ref).abs().max() <= 0.01 * ref.abs().max()
    # no activation, no bias
    A = torch.randn(128, 64, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(256, 64, generator=g).to(torch.bfloat16).cuda()
    Cf = torch.empty(128, 256, device="cuda")
    assert lib.ewf_mlp_gemm(_p(A), _p(B), None, _p(Cf), None, None, 128, 256, 64, 0, None) == 0
    torch.cuda.synchronize()
    ref = A.double() @ B.double().T
    assert (Cf.double() - ref).norm() / ref.norm() < 1e-6
    # shape checks are status codes
    assert lib.ewf_mlp_gemm(_p(A), _p(B), None, _p(Cf), None, None, 100, 256, 64, 0, None) == -1


def test_gemm_shapes_and_status(cuda_device):
    """The tcgen05 GEMM against an FP64 product of the same bf16 operands over its shape classes:
    256-wide tiles (N a multiple of 256) and 128-wide ones, a partial last k-stage (K = 32, 96,
    544: the tensor map's zero fill), many stages, the surrogate's output-layer shape, bias + GELU
    with every output, and a clean status afterwards."""
    import torch

    lib = load_library()
    g = torch.Generator(device="cpu").manual_seed(1)
    for M, N, K in ((128, 128, 32), (256, 384, 96), (384, 256, 512), (512, 12800, 512), (256, 512, 544),
                    (128, 640, 2048)):
        A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
        B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
        bias = torch.randn(N, generator=g).cuda()
        Cf = torch.empty(M, N, device="cuda")
        Cb = torch.empty(M, N, dtype=torch.bfloat16, device="cuda")
        pre = torch.empty(M, N, device="cuda")
        assert lib.ewf_mlp_gemm(_p(A), _p(B), _p(bias), _p(Cf), _p(Cb), _p(pre), M, N, K, 1, None) == 0
        torch.cuda.synchronize()
        assert lib.ewf_mlp_status() == 0
        ref_pre = A.double() @ B.double().T + bias.double()
        # fp32 accumulation: the relative error grows like sqrt(K) times the fp32 unit roundoff
        tol = 1e-6 * max(1.0, (K / 256) ** 0.5)
        err = ((pre.double() - ref_pre).norm() / ref_pre.norm()).item()
        assert err < tol, (M, N, K, err)
        ref = torch.nn.functional.gelu(ref_pre)
        assert (Cf.double() - ref).norm() / ref.norm() < tol
        assert (Cb.double() - ref).abs().max() <= 0.01 * ref.abs().max()
    # fp32-only output with two tiles per SM or more: the epilogue stages rows in shared memory and
    # writes them with TMA stores (both tile widths, bias + GELU applied in the staged path)
    for M, N, K, act in ((2048, 4864, 96, 1), (8192, 640, 512, 0), (4096, 12800, 512, 1)):
        A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
        B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
        bias = torch.randn(N, generator=g).cuda()
        Cf = torch.full((M, N), float("nan"), device="cuda")
        assert lib.ewf_mlp_gemm(_p(A), _p(B), _p(bias), _p(Cf), None, None, M, N, K, act, None) == 0
        torch.cuda.synchronize()
        assert lib.ewf_mlp_status() == 0
        ref = A.double() @ B.double().T + bias.double()
        if act:
            ref = torch.nn.functional.gelu(ref)
        tol = 1e-6 * max(1.0, (K / 256) ** 0.5)
        err = ((Cf.double() - ref).norm() / ref.norm()).item()
        assert err < tol, (M, N, K, err)


def test_gemm_wait_gives_up_and_next_launch_recovers(cuda_device):
    """Failure path of the GEMM's bounded waits: the test hook withholds the accumulator-ready
    signal of the first CTA's first tile (a signal nothing else gives), so the epilogue's wait
    runs out; the launch still ends, ewf_mlp_status reports it, and the next launch is exact."""
    import torch

    lib = load_library()
    g = torch.Generator(device="cpu").manual_seed(3)
    M, N, K = 256, 512, 128
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    Cf = torch.zeros(M, N, device="cuda")
    assert lib.ewf_mlp_status() == 0
    assert lib.ewf_mlp_test_hold(0, 20000) == 0
    try:
        assert lib.ewf_mlp_gemm(_p(A), _p(B), None, _p(Cf), None, None, M, N, K, 0, None) == 0
        st = lib.ewf_mlp_status()
    finally:
        assert lib.ewf_mlp_test_hold(-1, 0) == 0
    assert st == -2 and b"gave up" in lib.ewf_last_error()
    assert torch.isnan(Cf[:128, :256]).all(), "the held tile's outputs are marked invalid"
    assert lib.ewf_mlp_gemm(_p(A), _p(B), None, _p(Cf), None, None, M, N, K, 0, None) == 0
    assert lib.ewf_mlp_status() == 0
    ref = A.double() @ B.double().T
    assert (Cf.double() - ref).norm() / ref.norm() < 1e-6


def test_transpose_adam_and_gelu_grad(cuda_device):
    import torch

    lib = load_library()
    x = torch.randn(200, 333).to(torch.bfloat16).cuda()
    y = torch.empty(333, 200, dtype=torch.bfloat16, device="cuda")
    assert lib.ewf_mlp_transpose(_p(x), _p(y), 200, 333, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(y, x.T.contiguous())
    n = 1000
    w, m, v, gr = (torch.randn(n, device="cuda") for _ in range(4))
    m.abs_(); v.abs_()
    ref_w, ref_m, ref_v = w.double().clone(), m.double().clone(), v.double().clone()
    wb = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    assert lib.ewf_mlp_adam(_p(w), _p(m), _p(v), _p(gr), _p(wb), n, C.c_float(1e-2), C.c_float(0.9), C.c_float(0.999),
                            C.c_float(1e-8), 3, C.c_float(0.0), None) == 0
    torch.cuda.synchronize()
    g64 = gr.double()
    ref_m = 0.9 * ref_m + 0.1 * g64
    ref_v = 0.999 * ref_v + 0.001 * g64 * g64
    ref_w = ref_w - 1e-2 * (ref_m / (1 - 0.9 ** 3)) / ((ref_v / (1 - 0.999 ** 3)).sqrt() + 1e-8)
    assert (w.double() - ref_w).abs().max() < 1e-5
    assert torch.equal(wb, w.to(torch.bfloat16))
    pre = torch.randn(4096, device="cuda") * 3
    dy = torch.randn(4096, device="cuda").to(torch.bfloat16)
    dx = torch.empty(4096, dtype=torch.bfloat16, device="cuda")
    assert lib.ewf_mlp_gelu_grad(_p(dy), _p(pre), _p(dx), 4096, None) == 0
    torch.cuda.synchronize()
    ref = dy.double().cpu().numpy() * MO.gelu_grad(pre.double().cpu().numpy())
    assert np.abs(dx.double().cpu().numpy() - ref).max() <= 0.01 * np.abs(ref).max()


def test_mlp_gradients_match_fp64_oracle(cuda_device):
    import torch

    from elanfmt_gb300.surrogate import MLP

    sizes = [128, 128, 256, 128]
    net = MLP(sizes, seed=3)
    g = torch.Generator(device="cpu").manual_seed(1)
    X = torch.randn(128, 128, generator=g).to(torch.bfloat16).cuda()
    T = torch.randn(128, 128, generator=g).cuda()
    net.forward(X)
    loss = float(net.loss_grad(T))
    net.backward(128)
    torch.cuda.synchronize()
    w = net._work(128)
    Ws = [wb.double().cpu().numpy() for wb in net.Wb]
    bs = [b.double().cpu().numpy() for b in net.b]
    ref_loss, gW, gb = MO.loss_and_grads(X.double().cpu().numpy(), T.double().cpu().numpy(), Ws, bs)
    assert abs(loss - ref_loss) < 1e-2 * ref_loss
    for l in range(3):
        got = w["gW"][l].double().cpu().numpy()
        rel = np.linalg.norm(got - gW[l]) / np.linalg.norm(gW[l])
        cos = float((got * gW[l]).sum() / (np.linalg.norm(got) * np.linalg.norm(gW[l])))
        assert rel < 3e-2 and cos > 0.999, (l, rel, cos)
        gotb = w["gb"][l].double().cpu().numpy()
        assert np.linalg.norm(gotb - gb[l]) / np.linalg.norm(gb[l]) < 3e-2


def test_training_fits_a_smooth_map(cuda_device):
    """Training with the project's kernels reaches the loss a plain torch fp32 model of the same
    shape reaches with Adam on the same data and schedule."""
    import math

    import torch

    from elanfmt_gb300.surrogate import MLP

    g = torch.Generator(device="cpu").manual_seed(2)
    x = torch.rand(2048, 5, generator=g) * 2 - 1
    t = torch.linspace(0, 1, 256)
    Y = torch.tanh(2.0 * x[:, :1] + t[None, :] * x[:, 1:2]) * (1 + 0.5 * x[:, 2:3])
    Xp = torch.zeros(2048, 128)
    Xp[:, :5] = x
    Xg, Yg = Xp.to(torch.bfloat16).cuda(), Y.cuda()
    net = MLP([128, 256, 256, 256], seed=0, fan_in0=5)
    losses = net.train(Xg, Yg, steps=600, batch=256, lr=2e-3, log_every=100)
    # torch fp32 reference, same sizes, optimiser and schedule
    torch.manual_seed(0)
    ref = torch.nn.Sequential(torch.nn.Linear(5, 256), torch.nn.GELU(), torch.nn.Linear(256, 256), torch.nn.GELU(),
                              torch.nn.Linear(256, 256)).cuda()
    opt = torch.optim.Adam(ref.parameters(), lr=2e-3)
    xr, gr = x.cuda(), torch.Generator(device="cuda").manual_seed(0)
    for s in range(600):
        for q in opt.param_groups:
            q["lr"] = 2e-3 * 0.5 * (1 + math.cos(math.pi * s / 600))
        idx = torch.randint(0, 2048, (256,), device="cuda", generator=gr)
        loss = ((ref(xr[idx]) - Yg[idx]) ** 2).mean()
        opt.zero_grad()
        loss.backward()
        opt.step()
    with torch.no_grad():
        ref_loss = float(((ref(xr) - Yg) ** 2).mean())
    pred = net.predict(Xg)
    our_loss = float(((pred - Yg) ** 2).mean())
    assert losses[-1][1] < 0.05 * losses[0][1], losses
    assert our_loss < 10 * ref_loss + 1e-3, (our_loss, ref_loss)


def test_combine_matches_einsum(cuda_device):
    import torch

    lib = load_library()
    g = torch.Generator(device="cpu").manual_seed(5)
    for M, nout, nin, T in ((3, 18, 10, 700), (130, 18, 10, 256), (1, 1, 1, 1)):
        R = torch.randn(M, nout, nin, generator=g).cuda()
        G = torch.randn(M, nin, T, generator=g).cuda()
        out = torch.empty(M, nout, T, device="cuda")
        assert lib.ewf_mlp_combine(_p(R), _p(G), _p(out), M, nout, nin, T, None) == 0
        torch.cuda.synchronize()
        ref = torch.einsum("mof,mft->mot", R.double(), G.double())
        assert (out.double() - ref).abs().max() < 1e-5 * ref.abs().max()
    assert lib.ewf_mlp_combine(_p(R), _p(G), _p(out), M, 64, 64, T, None) == -1


def test_network_beats_nearest_neighbour(cuda_device):
    """A small surrogate study end to end (solver data, training, judging by the solver): the trained
    network's median relative L2 error on held-out sources is well below that of the method
    without it (the nearest training sample in the same features, mixed for the query's
    azimuth), and the solver's own traces honour the lateral symmetry the structure relies on."""
    from elanfmt_gb300 import surrogate as S

    r = S.study(train_runs=24, test_runs=8, n=96, nt=640, per_run=32, steps=1500, max_offset=5000.0, log=lambda *a: None)
    assert r["test_samples"] > 200 and r["test_samples_without_energy"] == 0
    assert r["symmetry_floor_rel_l2"]["median"] < 0.03, r["symmetry_floor_rel_l2"]
    assert r["surrogate_rel_l2"]["median"] < 0.12, r["surrogate_rel_l2"]
    assert r["network_gain_median"] > 1.4, (r["surrogate_rel_l2"], r["nearest_neighbour_rel_l2"])
    assert r["gf_sets_per_s"]["surrogate_over_fdtd_all"] > 100


def test_symmetry_floor_falls_with_resolution(cuda_device):
    """The solver's departure from the lateral symmetry (the floor of the structured surrogate)
    on one physical model at two resolutions: at these short offsets (up to 5 km) halving the
    cell size (twice the points per wavelength, twice the steps over the same window) lowers it
    by more than 30 %.  (At 1-12 km the floor hardly moves with the cell size: there it is set by
    what the absorbing boundaries return, not by the stencil.)"""
    from elanfmt_gb300 import surrogate as S

    r = S.symmetry_floor(cases=((0.5, 120.0), (0.5, 60.0)), sources=6, n120=96, per_run=32, max_offset=5000.0,
                         steps_at_half_hz=640, log=lambda *a: None)
    assert [(x["f0_hz"], x["dx_m"], x["n"]) for x in r] == [(0.5, 120.0, 96), (0.5, 60.0, 192)]
    assert all(x["gf_sets"] > 150 for x in r)
    assert r[1]["points_per_s_wavelength_at_f0"] == pytest.approx(2 * r[0]["points_per_s_wavelength_at_f0"])
    assert r[1]["median"] < 0.7 * r[0]["median"], r


def test_five_input_network_and_fallback(cuda_device):
    """The five-input form (source x, y, depth, receiver offset, azimuth -> 18 traces, no symmetry
    assumed) trained on the same small study: it beats its nearest-neighbour method, and with the
    solver as fallback no served GF set exceeds the 1e-3 bar."""
    from elanfmt_gb300 import surrogate as S

    r = S.study(train_runs=24, test_runs=8, n=96, nt=640, per_run=32, steps=1500, max_offset=5000.0,
                forms=("structured", "full"), log=lambda *a: None)
    f = r["full"]
    assert f["features"].startswith("source x, y, depth")
    assert f["surrogate_rel_l2"]["median"] < f["nearest_neighbour_rel_l2"]["median"], f
    for form in ("structured", "full"):
        assert r[form]["effective_max_rel_l2_served"] <= 1e-3
        assert r[form]["gf_sets_per_s"]["with_fallback"] > 0
