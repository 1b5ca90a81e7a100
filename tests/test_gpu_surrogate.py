"""The learned surrogate on the GPU: the BF16 tensor-core GEMM against torch
fp32 matmul, the network's forward pass and every gradient against the FP64
oracle (oracle/surrogate_ref.py, itself pinned by finite differences), the
window check, the fallback controller, training, and what the trained
network gains over the plain stencil."""
import ctypes as C

import numpy as np
import pytest

from oracle import surrogate_ref as R

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


# ---------------------------------------------------------------- GEMM
@pytest.mark.parametrize("M,N,K,trans_a,splits", [(100, 70, 50, False, 1), (64, 64, 32, True, 1),
                                                  (33, 200, 300, False, 1),
                                                  (20, 30, 1000, True, 4)])
def test_gemm_matches_torch(cuda, M, N, K, trans_a, splits):
    torch = _torch()
    from pyphasefield_gb300 import _lib as L
    g = torch.Generator().manual_seed(M * N + K)
    a = torch.randn(M, K, generator=g).to(torch.bfloat16)
    b = torch.randn(K, N, generator=g).to(torch.bfloat16)
    bias = torch.randn(N, generator=g)
    ref = a.double() @ b.double()
    y0 = torch.randn(M, N, generator=g)
    a_dev = (a.t().contiguous() if trans_a else a).to(cuda)
    sam, sak = (1, M) if trans_a else (K, 1)
    b_dev = b.to(cuda)
    y = y0.clone().to(cuda)
    s = torch.cuda.current_stream()
    use_bias = splits == 1
    L.call("ppf_sg_gemm", C.c_void_p(a_dev.data_ptr()), sam, sak, C.c_void_p(b_dev.data_ptr()), N,
           1, C.c_void_p(y.data_ptr()), N, C.c_void_p(bias.to(cuda).data_ptr()) if use_bias else None,
           1, M, N, K, splits, C.c_void_p(s.cuda_stream))
    torch.cuda.synchronize()
    expect = y0.double() + ref + (bias.double() if use_bias else 0)
    err = (y.cpu().double() - expect).abs().max().item()
    assert err <= 2e-5 * K ** 0.5 * expect.abs().max().item()


@pytest.mark.parametrize("M,N,K", [(4096, 128, 64), (4300, 200, 136), (8192, 384, 192),
                                   (5017, 72, 520)])
def test_tcgen05_gemm_matches_torch_and_mma_sync(cuda, M, N, K):
    """GEMMs with K-contiguous operands and at least 4096 rows run on tcgen05
    (accumulator in tensor memory): against torch in float64 and against the
    mma.sync kernel (ppf_sg_set_tensor_path(0)); ragged M and N tiles."""
    torch = _torch()
    from pyphasefield_gb300 import _lib as L
    g = torch.Generator().manual_seed(M + N + K)
    a = torch.randn(M, K, generator=g).to(torch.bfloat16)
    bt = torch.randn(N, K, generator=g).to(torch.bfloat16)  # B stored [n][k]
    bias = torch.randn(N, generator=g)
    expect = a.double() @ bt.double().t() + bias.double()
    ad, bd, biasd = a.to(cuda), bt.to(cuda), bias.to(cuda)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    try:
        for path in (1, 0):
            L.call("ppf_sg_set_tensor_path", path)
            y = torch.zeros(M, N, device=cuda)
            L.call("ppf_sg_gemm", C.c_void_p(ad.data_ptr()), K, 1, C.c_void_p(bd.data_ptr()), 1, K,
                   C.c_void_p(y.data_ptr()), N, C.c_void_p(biasd.data_ptr()), 0, M, N, K, 1, s)
            torch.cuda.synchronize()
            outs.append(y.cpu().double())
    finally:
        L.call("ppf_sg_set_tensor_path", 1)
    for y in outs:
        assert (y - expect).abs().max().item() <= 2e-5 * K ** 0.5 * expect.abs().max().item()
    assert (outs[0] - outs[1]).abs().max().item() <= 1e-5 * expect.abs().max().item()
    from pyphasefield_gb300 import _lib
    flags = C.c_int32(0)
    L.call("ppf_status_take", C.byref(flags))
    assert flags.value & 2 == 0  # no wait timed out


def test_gemm_rejects_bad_arguments(cuda):
    from pyphasefield_gb300 import _lib as L
    with pytest.raises(L.PpfError):
        L.call("ppf_sg_gemm", None, 1, 1, None, 1, 1, None, 1, None, 0, 4, 4, 4, 1, None)


# ---------------------------------------------------------------- network vs oracle
P, CH, E, NB = 4, 16, 32, 2
NORM = (0.5, 2.0, 0.4, 10.0)
SCALE = (3.0, 5.0)


def _tiny(cuda, seed=0, B=2, H=16, W=20):
    torch = _torch()
    from pyphasefield_gb300.surrogate import SurrogateNet
    rng = np.random.default_rng(seed)
    params = R.random_params(P, CH, E, NB, rng)
    for k in params:
        if k.startswith("b"):
            params[k] = rng.normal(0, 0.1, params[k].shape)
    net = SurrogateNet(P=P, C=CH, E=E, nblocks=NB, device=cuda, in_norm=NORM, delta_scale=SCALE)
    net.load_params(params)
    params = net.params_numpy()  # the fp32 values the GPU holds
    f_old = np.stack([rng.random((B, H, W)), 0.4 + 0.05 * rng.random((B, H, W))], axis=1)
    f_new = f_old + 0.02 * rng.normal(size=f_old.shape)
    f_old = f_old.astype(np.float32).astype(np.float64)
    f_new = f_new.astype(np.float32).astype(np.float64)
    pitch = (W + 31) // 32 * 32
    def dev(f):  # noqa: E306
        t = torch.full((B, 2, H, pitch), float("nan"), dtype=torch.float32)
        t[..., :W] = torch.from_numpy(f)
        return t.to(cuda)
    return net, params, f_old, f_new, dev(f_old), dev(f_new), (B, H, W, pitch)


@pytest.mark.parametrize("B,H,W,tc", [(2, 16, 20, 1), (1, 256, 256, 0), (1, 256, 256, 1)])
def test_forward_matches_oracle(cuda, B, H, W, tc):
    """4096 tokens (256^2 / 4^2) with tc = 1: the 1x1 convolutions run on
    tcgen05; the 40-token case and tc = 0 on mma.sync."""
    torch = _torch()
    from pyphasefield_gb300 import _lib as L
    net, params, f_old, _, d_old, _, shp = _tiny(cuda, B=B, H=H, W=W)
    L.call("ppf_sg_set_tensor_path", tc)
    try:
        out = net.forward(d_old, *shp, torch.cuda.current_stream()).cpu().double().numpy()
    finally:
        L.call("ppf_sg_set_tensor_path", 1)
    ref, _ = R.forward(params, f_old, P, NB, NORM, bf16_ops=True)
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 2e-3
    exact, _ = R.forward(params, f_old, P, NB, NORM, bf16_ops=False)
    assert np.linalg.norm(out - exact) / np.linalg.norm(exact) < 3e-2


def test_gradients_match_oracle(cuda):
    torch = _torch()
    net, params, f_old, f_new, d_old, d_new, shp = _tiny(cuda, seed=1)
    s = torch.cuda.current_stream()
    net.forward(d_old, *shp, s)
    loss = net.backward(d_old, d_new, *shp, s).item()
    grads = net.grads_numpy()
    l16, g16, _ = R.loss_and_grads(params, f_old, f_new, P, NB, NORM, SCALE, bf16_ops=True)
    l64, g64, _ = R.loss_and_grads(params, f_old, f_new, P, NB, NORM, SCALE, bf16_ops=False)
    assert loss == pytest.approx(l16, rel=2e-3)
    for k in g16:
        n16 = np.linalg.norm(g16[k])
        assert np.linalg.norm(grads[k] - g16[k]) <= 1e-2 * n16 + 1e-9, k
        assert np.linalg.norm(grads[k] - g64[k]) <= 6e-2 * np.linalg.norm(g64[k]) + 1e-9, k


def test_predict_applies_scaled_change(cuda):
    torch = _torch()
    net, params, f_old, _, d_old, _, shp = _tiny(cuda, seed=2)
    s = torch.cuda.current_stream()
    out_f = torch.zeros_like(d_old)
    net.predict(d_old, out_f, *shp, s)
    ref, _ = R.forward(params, f_old, P, NB, NORM, bf16_ops=True)
    B, H, W, _ = shp
    d = R.unpatch(ref, B, H, W, P)
    expect = np.clip(f_old + np.stack([d[:, 0] / SCALE[0], d[:, 1] / SCALE[1]], axis=1), 0, 1)
    got = out_f[..., :W].cpu().double().numpy()
    assert np.abs(got - expect).max() < 2e-3 * np.abs(d).max() / min(SCALE)


def test_adam_step_matches_formula(cuda):
    torch = _torch()
    net, params, _, _, d_old, d_new, shp = _tiny(cuda, seed=3)
    s = torch.cuda.current_stream()
    net.forward(d_old, *shp, s)
    net.backward(d_old, d_new, *shp, s)
    g = net.grads_numpy()
    net.adam(1e-2, s)
    w = net.params_numpy()
    for k in ("w_in", "b1_0", "dw1"):
        m = 0.1 * g[k] / 0.1
        v = 0.001 * g[k] ** 2 / 0.001
        expect = params[k] - 1e-2 * m / (np.sqrt(v) + 1e-8)
        np.testing.assert_allclose(w[k], expect, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(net.flat_b.float().cpu().numpy(),
                                  net.flat.to(torch.bfloat16).float().cpu().numpy())


# ---------------------------------------------------------------- window check
def test_residual_kernel(cuda):
    torch = _torch()
    from pyphasefield_gb300 import _lib as L
    from pyphasefield_gb300.surrogate import SurrogateNet
    net = SurrogateNet(P=4, C=8, E=8, nblocks=1, device=cuda)
    B, H, W, pitch, k = 2, 12, 20, 32, 16
    rng = np.random.default_rng(0)
    u, p, st = (rng.random((B, 2, H, W)) for _ in range(3))
    p[1, 1, 3, 4] = np.inf
    dev = []
    for a in (u, p, st):
        t = torch.full((B, 2, H, pitch), float("nan"), dtype=torch.float32)
        t[..., :W] = torch.from_numpy(a)
        dev.append(t.to(cuda))
    out = torch.full((B * 3,), 7.0, dtype=torch.float64, device=cuda)
    shape = net.shape(B, H, W, pitch)
    L.call("ppf_sg_residual", C.byref(shape), C.c_void_p(dev[0].data_ptr()),
           C.c_void_p(dev[1].data_ptr()), C.c_void_p(dev[2].data_ptr()), k,
           C.c_void_p(out.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    got = out.cpu().numpy().reshape(B, 3)
    u32, p32, s32 = (a.astype(np.float32).astype(np.float64) for a in (u, p, st))
    for b in range(B):
        r = k * (s32[b, 0] - p32[b, 0]) - (p32[b, 0] - u32[b, 0])
        assert got[b, 0] == pytest.approx((r * r).sum(), rel=1e-5)
        assert got[b, 1] == pytest.approx((p32[b, 0] ** 2).sum(), rel=1e-9)
    assert list(got[:, 2]) == [0.0, 1.0]


# ---------------------------------------------------------------- rollout controller
def _engine(H=64, seed=5):
    from pyphasefield_gb300.surrogate import make_sims
    sim = make_sims(1, H, seed)[0]
    sim.user_data["graph_chunk"] = 16
    sim.simulate(32)
    return sim


def test_rollout_falls_back_to_the_stencil(cuda):
    """A corrupted network (NaN weights) fails every check, so the rollout
    is the plain stencil, bit for bit."""
    from pyphasefield_gb300.surrogate import SurrogateNet, SurrogateRollout
    net = SurrogateNet(P=8, C=32, E=64, nblocks=1, device=cuda)
    net.flat.fill_(float("nan"))
    net.flat_b.fill_(float("nan"))
    a, b = _engine(), _engine()
    stats = SurrogateRollout(net, a, k=16, tol=1e-2, check_every=3).run(5)
    b.simulate(5 * 16)
    a.retrieve_fields_from_GPU()
    b.retrieve_fields_from_GPU()
    assert stats["segments"] == 2 and stats["rejected"] == 2 and stats["windows"] == 5
    assert stats["network_windows"] == 0 and stats["stencil_steps"] == 80
    assert a.time_step_counter == b.time_step_counter
    for fa, fb in zip(a.fields, b.fields):
        np.testing.assert_array_equal(fa.get_cells(), fb.get_cells())


def _stencil_steps(sim, x, n):
    torch = _torch()
    import ctypes
    y = torch.empty_like(x)
    sp = ctypes.c_void_p(sim._ppf_stream.cuda_stream)
    for i in range(n):
        sim._ppf_step([x[0, 0], x[0, 1]], [y[0, 0], y[0, 1]], 1, i, None, sp)
        x, y = y, x
    return x


def test_rollout_accepting_everything_chains_predictions(cuda):
    """With an infinite tolerance every segment is accepted: each is the
    network's windows followed by the stencil's verification window (graph
    and eager launches agree bit for bit)."""
    torch = _torch()
    from pyphasefield_gb300.surrogate import SurrogateNet, SurrogateRollout
    net = SurrogateNet(P=8, C=32, E=64, nblocks=2, device=cuda, delta_scale=(200.0, 500.0))
    a, b = _engine(), _engine()
    stats = SurrogateRollout(net, a, k=16, tol=np.inf, check_every=3).run(5)
    assert stats["rejected"] == 0 and stats["network_windows"] == 2 + 1
    assert stats["stencil_steps"] == 2 * 16 and len(stats["errors"]) == 2
    st = b._ppf_stream
    g = b._ppf_grid
    x = torch.stack([t for t in b._ppf_bufs[b._ppf_cur]])[None].contiguous()
    y = torch.empty_like(x)
    with torch.cuda.stream(st):
        for m in (3, 2):
            for _ in range(m - 1):
                net.predict(x, y, 1, g.kshape[0], g.kshape[1], g.pitch, st)
                x, y = y, x
            x = _stencil_steps(b, x, 16)
    st.synchronize()
    a.retrieve_fields_from_GPU()
    W = g.kshape[1]
    np.testing.assert_array_equal(a.fields[0].get_cells(), x[0, 0, :, :W].cpu().numpy())
    np.testing.assert_array_equal(a.fields[1].get_cells(), x[0, 1, :, :W].cpu().numpy())
    c = _engine()
    SurrogateRollout(net, c, k=16, tol=np.inf, check_every=3).run(5, use_graph=False)
    c.retrieve_fields_from_GPU()
    np.testing.assert_array_equal(a.fields[0].get_cells(), c.fields[0].get_cells())
    np.testing.assert_array_equal(a.fields[1].get_cells(), c.fields[1].get_cells())


def test_rollout_rejects_noise(cuda):
    from pyphasefield_gb300.surrogate import SurrogateNet, SurrogateRollout, make_sims
    net = SurrogateNet(P=8, C=16, E=16, nblocks=1, device=cuda)
    sim = make_sims(1, 64, 0)[0]
    sim.user_data["alpha"] = 0.3
    with pytest.raises(ValueError):
        SurrogateRollout(net, sim)


# ---------------------------------------------------------------- training and gain
@pytest.fixture(scope="module")
def trained(cuda):
    """A small network trained on stencil trajectories at 128^2 (k = 16)."""
    torch = _torch()
    from pyphasefield_gb300.surrogate import SurrogateNet, generate_trajectories, train
    data = generate_trajectories(12, 128, steps=512, k=16, seed=1, warm_steps=64)
    net = SurrogateNet(P=8, C=64, E=128, nblocks=4, device=cuda, seed=0)
    net.fit_normalisation(data, 128)
    hist = train(net, data, 128, iters=1500, batch=8, lr=2e-3, log_every=50)
    torch.cuda.synchronize()
    return net, data, hist


def test_training_reduces_loss(trained):
    _, _, hist = trained
    first = hist[0][1]
    last = np.mean([h[1] for h in hist[-3:]])
    assert np.isfinite(last)
    assert last < 0.25 * first, hist


def test_trained_network_beats_persistence_on_held_out(trained, cuda):
    """One-window prediction error on held-out trajectories: the network's
    k-step result against the stencil's, compared with predicting no change."""
    torch = _torch()
    from pyphasefield_gb300.surrogate import generate_trajectories
    net, _, _ = trained
    held = generate_trajectories(4, 128, steps=256, k=16, seed=99, warm_steps=64)
    s = torch.cuda.current_stream()
    n, m = held.shape[:2]
    err_net, err_id = [], []
    out = torch.empty_like(held[:, 0])
    for j in range(m - 1):
        net.predict(held[:, j].contiguous(), out, n, 128, 128, held.shape[-1], s)
        tgt = held[:, j + 1, 0, :, :128].double()
        err_net.append(((out[:, 0, :, :128].double() - tgt) ** 2).sum().item())
        err_id.append(((held[:, j, 0, :, :128].double() - tgt) ** 2).sum().item())
    print("held-out squared error net / persistence", np.sum(err_net) / np.sum(err_id))
    assert np.sum(err_net) < 0.3 * np.sum(err_id), (np.sum(err_net), np.sum(err_id))


def test_trained_network_gains_over_stencil_alone(trained, cuda):
    """What the network adds: under the same stencil check the trained
    network carries segments (each saving (check_every - 1) k stencil
    steps), while an untrained network of the same shape carries none."""
    from pyphasefield_gb300.surrogate import SurrogateNet, SurrogateRollout, make_sims, rel_l2
    net, _, _ = trained

    def run(network, tol):
        a, b = (make_sims(1, 128, 4242)[0] for _ in range(2))
        for s in (a, b):
            s.user_data["graph_chunk"] = 16
            s.simulate(64)
        b.retrieve_fields_from_GPU()
        start = b.fields[0].get_cells().copy()
        stats = SurrogateRollout(network, a, k=16, tol=tol, check_every=4).run(16)
        b.simulate(16 * 16)
        a.retrieve_fields_from_GPU()
        b.retrieve_fields_from_GPU()
        stats["persistence_error"] = rel_l2(start, b.fields[0].get_cells())
        return stats, rel_l2(a.fields[0].get_cells(), b.fields[0].get_cells())

    blank = SurrogateNet(P=8, C=64, E=128, nblocks=4, device=net.dev, seed=0)
    blank.in_norm, blank.delta_scale = net.in_norm, net.delta_scale
    probe, _ = run(blank, np.inf)
    tol = 0.5 * min(probe["errors"])  # half the untrained network's smallest check error
    stats, err = run(net, tol)
    stats0, err0 = run(blank, tol)
    print("tol", tol, "trained", stats, err, "untrained", stats0, err0)
    assert stats0["network_windows"] == 0 and err0 == 0.0
    assert stats["network_windows"] >= 6, stats
    assert stats["stencil_steps"] < 16 * 16
    # the rollout tracks the evolution far better than no evolution at all
    assert err < 0.5 * stats["persistence_error"], stats
