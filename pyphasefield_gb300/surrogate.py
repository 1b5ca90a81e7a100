"""Learned surrogate for Warren1995: a convolutional encoder-decoder that
advances the (phi, c) state by k stencil steps, trained on trajectories the
stencil itself generates, and run under a stencil check that falls back to
the stencil.

Network (every kernel is libppf_gb300's, see ppf_sg_* in
include/ppf_gb300.h; the GEMMs run on BF16 tensor cores with FP32
accumulation):

    patchify conv P x P / stride P (2 -> C)              implicit GEMM
    L x [depthwise 3x3 (C) -> 1x1 (C -> E) -> GELU -> 1x1 (E -> C)] + residual
    unpatchify conv (C -> 2 P^2): the normalised k-step change

The rollout controller (SurrogateRollout) runs windows of k steps in
segments; the last window of every segment is also advanced by the stencil
and the two results compared,

    e = || phi_net - phi_stencil ||_2 / || phi_net ||_2,

so the check measures the network's one-window error in the units of the
relative-L2 target. A segment whose check exceeds `tol` (or holds a
non-finite value) is recomputed by the stencil from its verified start.

A one-step residual k (S(u') - u') - (u' - u) was the first check tried
and is not usable for Warren1995 at k = 16: the interface is one to two
cells wide and moves about a cell per window, so the exact stencil
trajectory's own residual is as large as that of predicting no change at
all (both about 0.1-0.3 relative on phi at 512^2).

There is no counterpart in the reference; the engine it accelerates is
Engines/Warren1995.py:50-92 (the GB300 engine is Warren1995GB300).
"""
from __future__ import annotations

import ctypes as C
import gc
import math
import time

import numpy as np
import torch

from . import _lib as L
from .device import ptr

BF = torch.bfloat16
F32 = torch.float32


def _sp(stream) -> C.c_void_p:
    return C.c_void_p(stream.cuda_stream)


class SurrogateNet:
    """Parameters (one flat fp32 buffer with a bf16 mirror, gradient and Adam
    moments), activations and the forward / backward / Adam passes."""

    def __init__(self, P=16, C=192, E=384, nblocks=9, seed=0, device="cuda",
                 in_norm=(0.5, 2.0, 0.41, 20.0), delta_scale=(1.0, 1.0),
                 bounds=(0.0, 1.0, 0.0, 1.0)):
        self.P, self.C, self.E, self.L = int(P), int(C), int(E), int(nblocks)
        self.K = 2 * self.P * self.P
        self.in_norm = tuple(float(v) for v in in_norm)
        self.delta_scale = tuple(float(v) for v in delta_scale)
        # predicted phi and c stay in the model's physical range [0, 1]: an
        # overshoot would make the explicit stencil step unstable
        self.bounds = tuple(float(v) for v in bounds)
        self.dev = torch.device(device)
        spec = [("w_in", (self.C, self.K)), ("b_in", (self.C,)),
                ("w_out", (self.K, self.C)), ("b_out", (self.K,))]
        for l in range(self.L):
            spec += [(f"dw{l}", (self.C, 9)), (f"bdw{l}", (self.C,)), (f"w1_{l}", (self.E, self.C)),
                     (f"b1_{l}", (self.E,)), (f"w2_{l}", (self.C, self.E)), (f"b2_{l}", (self.C,))]
        self.spec = spec
        offs, o = {}, 0
        for name, shp in spec:
            offs[name] = o
            o += (math.prod(shp) + 63) // 64 * 64
        self.offs, self.size = offs, o
        self.flat = torch.zeros(o, dtype=F32, device=self.dev)
        self.flat_b = torch.zeros(o, dtype=BF, device=self.dev)
        self.flat_g = torch.zeros(o, dtype=F32, device=self.dev)
        self.flat_m1 = torch.zeros(o, dtype=F32, device=self.dev)
        self.flat_m2 = torch.zeros(o, dtype=F32, device=self.dev)
        view = lambda buf, n, s: buf[offs[n]:offs[n] + math.prod(s)].view(s)  # noqa: E731
        self.w = {n: view(self.flat, n, s) for n, s in spec}
        self.wb = {n: view(self.flat_b, n, s) for n, s in spec}
        self.g = {n: view(self.flat_g, n, s) for n, s in spec}
        self.init_params(seed)
        self.adam_step = 0
        self._shape_key = None

    # ------------------------------------------------------------ parameters
    @property
    def n_params(self) -> int:
        return sum(math.prod(s) for _, s in self.spec)

    def init_params(self, seed=0):
        g = torch.Generator().manual_seed(int(seed))
        init = {}
        for n, s in self.spec:
            if n.startswith("b"):
                init[n] = torch.zeros(s)
            elif n.startswith("dw"):
                init[n] = torch.randn(*s, generator=g) / 3.0
            elif n.startswith("w2_") or n == "w_out":
                init[n] = torch.randn(*s, generator=g) * (0.1 / math.sqrt(s[1]))
            else:
                init[n] = torch.randn(*s, generator=g) / math.sqrt(s[1])
        self.load_params(init)

    def load_params(self, params: dict):
        """Set the fp32 weights (and their bf16 mirror) from arrays."""
        for n, s in self.spec:
            self.w[n].copy_(torch.as_tensor(np.asarray(params[n]), dtype=F32).reshape(s))
        self.flat_b.copy_(self.flat.to(BF))

    def params_numpy(self) -> dict:
        return {n: self.w[n].detach().cpu().numpy().astype(np.float64) for n, _ in self.spec}

    def grads_numpy(self) -> dict:
        return {n: self.g[n].detach().cpu().numpy().astype(np.float64) for n, _ in self.spec}

    def save(self, path):
        np.savez(path, P=self.P, C=self.C, E=self.E, L=self.L, in_norm=self.in_norm,
                 delta_scale=self.delta_scale, bounds=self.bounds, **self.params_numpy())

    @classmethod
    def load(cls, path, device="cuda"):
        z = np.load(path)
        net = cls(P=int(z["P"]), C=int(z["C"]), E=int(z["E"]), nblocks=int(z["L"]),
                  device=device, in_norm=tuple(z["in_norm"]), delta_scale=tuple(z["delta_scale"]),
                  bounds=tuple(z["bounds"]) if "bounds" in z.files else (0.0, 1.0, 0.0, 1.0))
        net.load_params({n: z[n] for n, _ in net.spec})
        return net

    def fit_normalisation(self, data: torch.Tensor, W: int):
        """Input offsets/scales and change scales from snapshot data
        [n_traj, n_snap, 2, H, pitch] (interior columns [:W])."""
        x = data[..., :W]
        c = x[:, :, 1].double()
        self.in_norm = (0.5, 2.0, float(c.mean()), 1.0 / max(float(c.std()), 1e-12))
        del c
        sd = []
        for ch in (0, 1):
            d = (x[:, 1:, ch] - x[:, :-1, ch]).double()
            sd.append(1.0 / max(float(d.std()), 1e-12))
            del d
        self.delta_scale = tuple(sd)

    # ------------------------------------------------------------ buffers
    def shape(self, B, H, W, pitch) -> L.PpfSgShape:
        s = L.PpfSgShape()
        s.B, s.H, s.W, s.pitch, s.P, s.C, s.E = B, H, W, pitch, self.P, self.C, self.E
        s.s0, s.s1 = self.delta_scale
        s.in_off0, s.in_sc0, s.in_off1, s.in_sc1 = self.in_norm
        s.lo0, s.hi0, s.lo1, s.hi1 = self.bounds
        return s

    def _alloc(self, B, H, W):
        key = (B, H, W)
        if self._shape_key == key:
            return
        if H % self.P or W % self.P:
            raise ValueError(f"grid {H}x{W} is not a multiple of the patch size {self.P}")
        T = B * (H // self.P) * (W // self.P)
        z = lambda n, dt=F32: torch.empty(T, n, dtype=dt, device=self.dev)  # noqa: E731
        Lb = self.L
        self.a = {
            "y": [z(self.C) for _ in range(Lb + 1)], "yb": [z(self.C, BF) for _ in range(Lb + 1)],
            "h": [z(self.C) for _ in range(Lb)], "hb": [z(self.C, BF) for _ in range(Lb)],
            "pre": [z(self.E) for _ in range(Lb)], "act": [z(self.E, BF) for _ in range(Lb)],
            "out": z(self.K), "dout": z(self.K, BF), "dy": z(self.C), "dy2": z(self.C),
            "dyb": z(self.C, BF), "dpre": z(self.E, BF), "dh": z(self.C), "dhb": z(self.C, BF),
            "loss": torch.zeros(1, dtype=torch.float64, device=self.dev)}
        self._shape_key = key

    # ------------------------------------------------------------ passes
    def forward(self, fields, B, H, W, pitch, stream):
        """fields [B, 2, H, pitch] float32 -> out [tokens, 2 P^2] (the
        normalised change)."""
        self._alloc(B, H, W)
        s = self.shape(B, H, W, pitch)
        sp = _sp(stream)
        a, w, wb = self.a, self.w, self.wb
        L.call("ppf_sg_patch_fwd", C.byref(s), ptr(fields), ptr(wb["w_in"]), ptr(w["b_in"]),
               ptr(a["y"][0]), ptr(a["yb"][0]), sp)
        for l in range(self.L):
            L.call("ppf_sg_block_fwd", C.byref(s), ptr(a["y"][l]), ptr(w[f"dw{l}"]),
                   ptr(w[f"bdw{l}"]), ptr(a["h"][l]), ptr(a["hb"][l]), ptr(wb[f"w1_{l}"]),
                   ptr(w[f"b1_{l}"]), ptr(a["pre"][l]), ptr(a["act"][l]), ptr(wb[f"w2_{l}"]),
                   ptr(w[f"b2_{l}"]), ptr(a["y"][l + 1]), ptr(a["yb"][l + 1]), sp)
        L.call("ppf_sg_head_fwd", C.byref(s), ptr(a["yb"][self.L]), ptr(wb["w_out"]),
               ptr(w["b_out"]), ptr(a["out"]), sp)
        return a["out"]

    def backward(self, f_old, f_new, B, H, W, pitch, stream):
        """After forward(f_old): MSE against the normalised change
        f_new - f_old (device scalar a['loss']), gradients into self.g."""
        s = self.shape(B, H, W, pitch)
        sp = _sp(stream)
        a, w, wb, g = self.a, self.w, self.wb, self.g
        with torch.cuda.stream(stream):
            a["loss"].zero_()
            self.flat_g.zero_()
        L.call("ppf_sg_mse", C.byref(s), ptr(a["out"]), ptr(f_old), ptr(f_new), ptr(a["dout"]),
               ptr(a["loss"]), sp)
        L.call("ppf_sg_head_bwd", C.byref(s), ptr(a["yb"][self.L]), ptr(wb["w_out"]),
               ptr(a["dout"]), ptr(g["w_out"]), ptr(g["b_out"]), ptr(a["dy"]), ptr(a["dyb"]), sp)
        dy, dy2 = a["dy"], a["dy2"]
        for l in reversed(range(self.L)):
            L.call("ppf_sg_block_bwd", C.byref(s), ptr(a["y"][l]), ptr(a["hb"][l]),
                   ptr(a["pre"][l]), ptr(a["act"][l]), ptr(wb[f"w1_{l}"]), ptr(wb[f"w2_{l}"]),
                   ptr(w[f"dw{l}"]), ptr(dy), ptr(a["dyb"]), ptr(a["dpre"]), ptr(a["dh"]),
                   ptr(a["dhb"]), ptr(dy2), ptr(g[f"w1_{l}"]), ptr(g[f"b1_{l}"]),
                   ptr(g[f"w2_{l}"]), ptr(g[f"b2_{l}"]), ptr(g[f"dw{l}"]), ptr(g[f"bdw{l}"]), sp)
            dy, dy2 = dy2, dy
            L.call("ppf_sg_cast_bf16", ptr(dy), ptr(a["dyb"]), C.c_longlong(dy.numel()), sp)
        L.call("ppf_sg_patch_bwd_weight", C.byref(s), ptr(f_old), ptr(a["dyb"]), ptr(g["w_in"]),
               ptr(g["b_in"]), sp)
        return a["loss"]

    def adam(self, lr, stream, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0):
        """One Adam step over every parameter (one launch), refreshing the
        bf16 mirror."""
        self.adam_step += 1
        L.call("ppf_sg_adam", ptr(self.flat), ptr(self.flat_b), ptr(self.flat_g), ptr(self.flat_m1),
               ptr(self.flat_m2), C.c_longlong(self.size), C.c_float(lr), C.c_float(b1),
               C.c_float(b2), C.c_float(eps), self.adam_step, C.c_float(weight_decay), _sp(stream))

    def predict(self, fields, out_fields, B, H, W, pitch, stream):
        """out_fields = fields advanced k steps by the network (interior
        columns; padding columns are left as they are)."""
        self.forward(fields, B, H, W, pitch, stream)
        s = self.shape(B, H, W, pitch)
        L.call("ppf_sg_apply", C.byref(s), ptr(self.a["out"]), ptr(fields), ptr(out_fields),
               _sp(stream))

    def flops_per_token(self) -> int:
        """Forward FLOPs (2 x multiply-adds) per token: patch, blocks, head."""
        per_block = self.C * 9 + 2 * self.C * self.E
        return 2 * (2 * self.K * self.C + self.L * per_block)


# ---------------------------------------------------------------- data
def seeded_state(H, W, rng, c0=0.40783, nuclei=(1, 8), radius=5.0):
    """phi = 1 (liquid) with 1..8 solid disks (phi = 0) of `radius` cells at
    random positions, c = c0 + U(-1e-3, 1e-3)."""
    phi = np.ones((H, W))
    yy, xx = np.mgrid[0:H, 0:W]
    for _ in range(int(rng.integers(nuclei[0], nuclei[1] + 1))):
        cy, cx = rng.uniform(8, H - 8), rng.uniform(8, W - 8)
        phi[(yy - cy) ** 2 + (xx - cx) ** 2 < radius ** 2] = 0.0
    return phi, c0 + rng.uniform(-1e-3, 1e-3, (H, W))


def make_sims(n, H, seed, dT=(5.0, 40.0), c0=0.40783):
    """n initialised Warren1995GB300 engines (noise off) from random nuclei
    and undercooling dT below the liquidus of c0."""
    from .engines import Warren1995GB300
    from .ensemble import warren_liquidus
    rng = np.random.default_rng(seed)
    t_ref = warren_liquidus(c0, Warren1995GB300.DEFAULTS)
    sims = []
    for i in range(n):
        sim = Warren1995GB300(dimensions=[H, H], dx=4.6e-8, boundary_conditions="NEUMANN",
                              user_data={"T": float(t_ref - rng.uniform(*dT)), "alpha": 0.0,
                                         "seed": int(seed) * 100003 + i})
        sim.initialize_fields_and_imported_data()
        phi, c = seeded_state(H, H, rng, c0=c0)
        sim.fields[0].data[1:-1, 1:-1] = phi
        sim.fields[1].data[1:-1, 1:-1] = c
        sims.append(sim)
    return sims


def generate_trajectories(n_traj, H, steps, k, seed=0, warm_steps=64, dT=(5.0, 40.0)):
    """Stencil-generated training data: n_traj Warren1995 runs stepped
    together by the ensemble launch; snapshots every k steps after
    `warm_steps`. Returns a device tensor [n_traj, n_snap, 2, H, pitch]."""
    from .ensemble import Ensemble
    sims = make_sims(n_traj, H, seed, dT)
    ens = Ensemble(sims, graph_chunk=k)
    if warm_steps:
        ens.simulate(warm_steps)
    n_snap = steps // k + 1
    pitch = sims[0]._ppf_grid.pitch
    data = torch.empty((n_traj, n_snap, 2, H, pitch), dtype=F32, device=sims[0]._ppf_grid.device)
    for j in range(n_snap):
        if j:
            ens.simulate(k)
        with torch.cuda.stream(ens.stream):
            for i, s in enumerate(sims):
                data[i, j, 0].copy_(s._ppf_bufs[s._ppf_cur][0])
                data[i, j, 1].copy_(s._ppf_bufs[s._ppf_cur][1])
    ens.synchronize()
    return data


def train(net, data, W, iters=2000, batch=8, lr=1e-3, seed=0, log_every=100, stream=None,
          warmup=100):
    """Adam on random (trajectory, window) pairs with linear warm-up and
    cosine decay; returns [(iteration, loss)]."""
    stream = stream or torch.cuda.current_stream()
    n_traj, n_snap, _, H, pitch = data.shape
    gen = torch.Generator(device=data.device).manual_seed(int(seed))
    f_old = torch.empty((batch, 2, H, pitch), dtype=F32, device=data.device)
    f_new = torch.empty_like(f_old)
    hist = []
    for it in range(iters):
        with torch.cuda.stream(stream):
            ti = torch.randint(0, n_traj, (batch,), generator=gen, device=data.device)
            wi = torch.randint(0, n_snap - 1, (batch,), generator=gen, device=data.device)
            f_old.copy_(data[ti, wi])
            f_new.copy_(data[ti, wi + 1])
        rate = lr * min(1.0, (it + 1) / warmup) * 0.5 * (1 + math.cos(math.pi * it / max(1, iters)))
        net.forward(f_old, batch, H, W, pitch, stream)
        loss = net.backward(f_old, f_new, batch, H, W, pitch, stream)
        net.adam(rate, stream)
        if it % log_every == 0 or it == iters - 1:
            hist.append((it, float(loss.item())))
    return hist


# ---------------------------------------------------------------- rollout
class SurrogateRollout:
    """Surrogate time stepping of one Warren1995GB300 engine (2-D float32,
    alpha = 0) in windows of k steps, verified by the stencil.

    Windows run in segments of `check_every`. In a segment the network
    advances the state window after window; for the segment's last window
    the stencil also advances k steps from the same state, and the two
    results are compared (relative L2 on phi, plus a non-finite count). If
    the network's last window is within `tol` of the stencil's, the segment
    is accepted and continues from the stencil's result; otherwise the whole
    segment is recomputed by the stencil from its verified starting state.
    Every segment is one CUDA graph launch and one host read of the check."""

    def __init__(self, net: SurrogateNet, sim, k=16, tol=1e-2, check_every=8):
        if not sim._ppf_ready():
            sim._begun_simulation = True
            sim.just_before_simulating()
        if float(sim.user_data.get("alpha", 0.0)) != 0.0:
            raise ValueError("the surrogate models the noise-free dynamics (alpha = 0)")
        if sim._ppf_dtype != torch.float32:
            raise ValueError("the surrogate runs on float32 engines")
        self.net, self.sim, self.k, self.tol = net, sim, int(k), float(tol)
        self.n = max(1, int(check_every))
        g = sim._ppf_grid
        self.H, self.W = g.kshape
        self.pitch = g.pitch
        dev = g.device
        self.stream = sim._ppf_stream
        z = lambda *s: torch.zeros(*s, 2, self.H, self.pitch, dtype=F32, device=dev)  # noqa: E731
        self.states = z(self.n + 1, 1)
        self.ref, self.tmp = z(1), z(1)
        self.res = torch.zeros(3, dtype=torch.float64, device=dev)
        self.res_host = torch.zeros(3, dtype=torch.float64, pin_memory=True)
        self.shape = net.shape(1, self.H, self.W, self.pitch)
        self.graphs = {}
        self.reset_stats()

    def reset_stats(self):
        self.stats = {"windows": 0, "segments": 0, "rejected": 0, "network_windows": 0,
                      "stencil_steps": 0, "errors": []}

    @staticmethod
    def _bufs(t):
        return [t[0, 0], t[0, 1]]

    def _verified_result(self):
        return self.tmp if self.k % 2 == 0 else self.ref

    def _segment(self, m, step0):
        """Network windows states[j] -> states[j+1] for j < m; the stencil's
        k steps from states[m-1]; their comparison into res."""
        sp = _sp(self.stream)
        for j in range(m):
            self.net.predict(self.states[j], self.states[j + 1], 1, self.H, self.W, self.pitch,
                             self.stream)
        src = self._bufs(self.states[m - 1])
        for i in range(self.k):
            dst = self._bufs(self.ref if i % 2 == 0 else self.tmp)
            self.sim._ppf_step(src, dst, 1, step0 + i, None, sp)
            src = dst
        out = self._verified_result()
        # with u = pred the check kernel's sums are ||stepped - pred||^2, ||pred||^2
        L.call("ppf_sg_residual", C.byref(self.shape), ptr(self.states[m]), ptr(self.states[m]),
               ptr(out), 1, ptr(self.res), sp)

    def _graph(self, m):
        g = self.graphs.get(m)
        if g is not None:
            return g
        self.net._alloc(1, self.H, self.W)
        sp = _sp(self.stream)
        gc_was = gc.isenabled()
        gc.disable()  # no pinned-buffer frees while capturing
        exec_ = C.c_void_p()
        try:
            L.call("ppf_graph_begin", sp)
            try:
                self._segment(m, 0)
            finally:
                L.call("ppf_graph_end", sp, C.byref(exec_))
        finally:
            if gc_was:
                gc.enable()
        self.graphs[m] = exec_
        return exec_

    def prepare(self, windows: int):
        """Capture the segment graphs a run of `windows` windows uses."""
        if windows >= self.n:
            self._graph(self.n)
        if windows % self.n:
            self._graph(windows % self.n)

    def run(self, windows: int, use_graph=True):
        """Advance the engine windows x k steps. Returns the statistics."""
        sim, s = self.sim, self.stream
        sp = _sp(s)
        with torch.cuda.stream(s):
            for j in (0, 1):
                self.states[0, 0, j].copy_(sim._ppf_bufs[sim._ppf_cur][j])
        left = int(windows)
        while left > 0:
            m = min(self.n, left)
            step0 = sim.time_step_counter
            if use_graph:
                L.call("ppf_graph_launch", self._graph(m), sp)
            else:
                self._segment(m, step0 + (m - 1) * self.k)
            with torch.cuda.stream(s):
                self.res_host.copy_(self.res, non_blocking=True)
            s.synchronize()
            num, den, bad = (float(v) for v in self.res_host)
            err = math.sqrt(num) / math.sqrt(den) if den > 0 else math.inf
            self.stats["errors"].append(err)
            self.stats["segments"] += 1
            if bad == 0 and err <= self.tol:
                with torch.cuda.stream(s):
                    self.states[0].copy_(self._verified_result())
                self.stats["network_windows"] += m - 1
                self.stats["stencil_steps"] += self.k
            else:  # the segment is recomputed by the stencil
                cur = sim._ppf_bufs[sim._ppf_cur]
                with torch.cuda.stream(s):
                    for j in (0, 1):
                        cur[j].copy_(self.states[0, 0, j])
                sim._ppf_advance(m * self.k, step0)
                cur = sim._ppf_bufs[sim._ppf_cur]
                with torch.cuda.stream(s):
                    for j in (0, 1):
                        self.states[0, 0, j].copy_(cur[j])
                self.stats["rejected"] += 1
                self.stats["stencil_steps"] += m * self.k
            self.stats["windows"] += m
            sim.time_step_counter += m * self.k
            left -= m
        with torch.cuda.stream(s):
            for j in (0, 1):
                sim._ppf_bufs[sim._ppf_cur][j].copy_(self.states[0, 0, j])
        return self.stats

    def __del__(self):
        try:
            for g in self.graphs.values():
                L.call("ppf_graph_destroy", g)
        except Exception:
            pass


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def evaluate(net, n_eval=4, H=512, windows=64, k=16, seed=10_000, tol=1e-2, check_every=8,
             warm_steps=64):
    """Held-out comparison against the plain stencil to the same simulated
    time. Each held-out engine is made twice (identical seeds), warmed up by
    `warm_steps` stencil steps, then advanced windows x k steps by (a) the
    stencil (CUDA-graph chunks of k) and (b) the surrogate rollout; wall
    times are taken with the device synchronised on both sides."""
    cases = []
    for i in range(n_eval):
        st = make_sims(1, H, seed + i)[0]
        su = make_sims(1, H, seed + i)[0]
        for s in (st, su):
            s.user_data["graph_chunk"] = k
            s.simulate(warm_steps)
        ro = SurrogateRollout(net, su, k=k, tol=tol, check_every=check_every)
        ro.prepare(windows)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st.simulate(windows * k)
        st.synchronize()
        t_st = time.perf_counter() - t0
        ro.reset_stats()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stats = ro.run(windows)
        su.synchronize()
        t_su = time.perf_counter() - t0
        st.retrieve_fields_from_GPU()
        su.retrieve_fields_from_GPU()
        cases.append({
            "phi_rel_l2": rel_l2(su.fields[0].get_cells(), st.fields[0].get_cells()),
            "c_rel_l2": rel_l2(su.fields[1].get_cells(), st.fields[1].get_cells()),
            "stencil_s": t_st, "surrogate_s": t_su,
            "segments": stats["segments"], "rejected": stats["rejected"],
            "network_windows": stats["network_windows"], "stencil_steps": stats["stencil_steps"],
            "max_check_error": max(stats["errors"]) if stats["errors"] else 0.0})
    sp = [c["stencil_s"] / c["surrogate_s"] for c in cases]
    return {"cases": cases, "speedup_min": min(sp), "speedup_mean": float(np.mean(sp)),
            "phi_rel_l2_max": max(c["phi_rel_l2"] for c in cases),
            "rejected_frac": sum(c["rejected"] for c in cases) / sum(c["segments"] for c in cases)}


def time_predict(net, H, reps=50):
    """Device time (ms) of one graph-launched B = 1 prediction at H x H."""
    pitch = (H + 31) // 32 * 32
    s = torch.cuda.Stream()
    x = torch.zeros((1, 2, H, pitch), dtype=F32, device=net.dev)
    x[:, 0] = 1.0
    x[:, 1] = net.in_norm[2]
    y = torch.empty_like(x)
    net._alloc(1, H, H)
    net.predict(x, y, 1, H, H, pitch, s)
    sp = _sp(s)
    exec_ = C.c_void_p()
    gc_was = gc.isenabled()
    gc.disable()
    try:
        L.call("ppf_graph_begin", sp)
        try:
            net.predict(x, y, 1, H, H, pitch, s)
        finally:
            L.call("ppf_graph_end", sp, C.byref(exec_))
    finally:
        if gc_was:
            gc.enable()
    try:
        for _ in range(3):
            L.call("ppf_graph_launch", exec_, sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            L.call("ppf_graph_launch", exec_, sp)
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps
    finally:
        L.call("ppf_graph_destroy", exec_)


def gemm_table(shapes=((1024, 384, 192), (8192, 384, 192), (8192, 512, 192), (65536, 384, 192),
                       (65536, 192, 384), (65536, 512, 512), (131072, 384, 192)), reps=20):
    """TFLOP/s of ppf_sg_gemm (K-contiguous bf16 operands, fp32 output) on
    the tcgen05 path and on mma.sync, CUDA events over `reps` launches after
    three warm-up launches; one dict per shape."""
    dev = torch.device("cuda")
    s = torch.cuda.current_stream()
    sp = _sp(s)
    rows = []
    try:
        for M, N, K in shapes:
            a = torch.randn(M, K, device=dev).to(BF)
            b = torch.randn(N, K, device=dev).to(BF)
            y = torch.zeros(M, N, device=dev)
            row = {"M": M, "N": N, "K": K}
            for path, name in ((1, "tcgen05"), (0, "mma_sync")):
                L.call("ppf_sg_set_tensor_path", path)

                def run():
                    L.call("ppf_sg_gemm", ptr(a), K, 1, ptr(b), 1, K, ptr(y), N, None, 0, M, N, K,
                           1, sp)

                for _ in range(3):
                    run()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(s)
                for _ in range(reps):
                    run()
                e1.record(s)
                e1.synchronize()
                row[name] = 2 * M * N * K / (e0.elapsed_time(e1) / reps / 1e3) / 1e12
            rows.append(row)
    finally:
        L.call("ppf_sg_set_tensor_path", 1)
    return rows


def held_out_error_ratio(net, held) -> float:
    """Sum over held-out windows of the network's squared phi error against
    the stencil, over the same for predicting no change."""
    s = torch.cuda.current_stream()
    n, m, _, H, pitch = held.shape
    out = torch.empty_like(held[:, 0])
    e_net = e_id = 0.0
    for j in range(m - 1):
        net.predict(held[:, j].contiguous(), out, n, H, H, pitch, s)
        tgt = held[:, j + 1, 0, :, :H].double()
        e_net += float(((out[:, 0, :, :H].double() - tgt) ** 2).sum())
        e_id += float(((held[:, j, 0, :, :H].double() - tgt) ** 2).sum())
    return e_net / e_id


def main(argv=None):
    """Train the surrogate on stencil trajectories and evaluate it on
    held-out seeds; prints one JSON summary line."""
    import argparse
    import json
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--k", type=int, default=16, help="stencil steps per network call")
    ap.add_argument("--trajectories", type=int, default=32)
    ap.add_argument("--steps", type=int, default=1024, help="steps per training trajectory")
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--patch", type=int, default=16)
    ap.add_argument("--channels", type=int, default=192)
    ap.add_argument("--expand", type=int, default=384)
    ap.add_argument("--blocks", type=int, default=9)
    ap.add_argument("--windows", type=int, default=64)
    ap.add_argument("--tol", type=float, default=1e-2)
    ap.add_argument("--check-every", type=int, default=8)
    ap.add_argument("--eval", type=int, default=2, help="held-out engines (0: training only)")
    ap.add_argument("--save", default=None, help="write the trained parameters (.npz)")
    ap.add_argument("--mma-sync", action="store_true",
                    help="run every GEMM on mma.sync (default: tcgen05 for the large "
                         "K-contiguous ones)")
    ap.add_argument("--gemm-table", action="store_true",
                    help="time the GEMM kernels at the network's shapes instead")
    a = ap.parse_args(argv)
    if a.gemm_table:
        for row in gemm_table():
            print(json.dumps(row), flush=True)
        return
    L.call("ppf_sg_set_tensor_path", 0 if a.mma_sync else 1)
    H, k = a.grid, a.k
    t0 = time.perf_counter()
    data = generate_trajectories(a.trajectories, H, a.steps, k, seed=1, warm_steps=64)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = SurrogateNet(P=a.patch, C=a.channels, E=a.expand, nblocks=a.blocks, seed=0)
    net.fit_normalisation(data, H)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = train(net, data, H, iters=a.iters, batch=a.batch, lr=a.lr,
                 log_every=max(1, a.iters // 10))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del data
    ratio, ev = None, None
    if a.eval > 0:
        held = generate_trajectories(2, H, 1024, k, seed=77, warm_steps=64)
        ratio = held_out_error_ratio(net, held)
        del held
    ms = time_predict(net, H)
    flops = (H // a.patch) ** 2 * net.flops_per_token()
    if a.eval > 0:
        ev = evaluate(net, n_eval=a.eval, H=H, windows=a.windows, k=k, tol=a.tol,
                      check_every=a.check_every)
    if a.save:
        net.save(a.save)
    tokens = a.batch * (H // a.patch) ** 2
    print(json.dumps({
        "grid": H, "k": k, "params": net.n_params,
        "tensor_path": "mma.sync" if a.mma_sync else "tcgen05 (K-contiguous, >= 4096 rows) + mma.sync",
        "net": {"patch": a.patch, "channels": a.channels, "expand": a.expand, "blocks": a.blocks},
        "data": {"trajectories": a.trajectories, "steps": a.steps, "seconds": round(t_data, 3),
                 "cell_updates": a.trajectories * (a.steps + 64) * H * H},
        "train": {"iters": a.iters, "batch": a.batch, "seconds": round(t_train, 3),
                  "ms_per_iter": round(1e3 * t_train / a.iters, 3),
                  "tflops": round(3 * tokens * net.flops_per_token() * a.iters / t_train / 1e12, 2),
                  "loss_first": hist[0][1], "loss_last": hist[-1][1]},
        "held_out_sq_error_vs_no_change": ratio,
        "predict": {"ms": round(ms, 4), "gflop": round(flops / 1e9, 3),
                    "tflops": round(flops / ms / 1e9, 2)},
        "eval": ev}))


if __name__ == "__main__":
    main()
