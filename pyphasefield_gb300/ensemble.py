"""Batched ensembles: many Warren1995 / Allen-Cahn engines advanced together.

The reference runs one Simulation at a time; an ensemble here is a list of
ordinary engine instances (each with its own fields, parameters and grid
size) whose device buffers are stepped together, a chunk of `graph_chunk`
steps per `ppf_ensemble_run_f32` call captured in a CUDA graph: one launch
per step over every member, or for four- and eight-row bands one persistent
cooperative launch per chunk (the CTAs meet at a bounded grid barrier
between steps). The rows per warp band, the bands per warp and the launch
kind are picked by the autotuner for the ensemble's mix of member sizes
(cached per mix and device). Afterwards each member is an ordinary
engine again: retrieve_fields_from_GPU, save_simulation etc. work on it.

`make_config_ensemble` builds the benchmark ensemble: n members whose square
sides are drawn log-uniform in [128, 1024]; even members are Warren1995 at
T = T_liquidus(c0) - dT with dT ~ U[5, 40] K and a solid nucleus at a random
position, odd members Allen-Cahn (reference defaults M=0.1, eps=1, W=1) with a
phi = 1 nucleus at a random position.
"""
from __future__ import annotations

import ctypes as C
import gc

import numpy as np
import torch

from . import _lib as L
from .device import ptr, tiling_struct
from .engines import CahnAllenGB300, Warren1995GB300


def warren_liquidus(c0: float, ud: dict) -> float:
    """Liquidus temperature of composition c0 in the Warren1995 model's own
    ideal-solution thermodynamics: with k_A = exp(v_m L_A (1/T - 1/T_mA)/R)
    and k_B = exp(v_m L_B (1/T - 1/T_mB)/R) the equilibrium liquid
    composition is c_L = (1 - k_A) / (k_B - k_A) (equal diffusion and grand
    potentials of phi = 0 and phi = 1 in the free energy whose phi-derivatives
    are the engine's H_A, H_B). Solved for T by bisection between the pure
    melting points."""
    vr = ud["v_m"] / ud["R"]

    def c_liquid(T):
        ka = np.exp(vr * ud["L_A"] * (1 / T - 1 / ud["T_mA"]))
        kb = np.exp(vr * ud["L_B"] * (1 / T - 1 / ud["T_mB"]))
        return (1 - ka) / (kb - ka)

    lo, hi = ud["T_mB"] + 1e-6, ud["T_mA"] - 1e-6  # c_L falls from ~1 to ~0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if c_liquid(mid) > c0:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def make_config_ensemble(n: int = 64, seed: int = 0, side_range=(128, 1024), c0=0.40783,
                         dT_range=(5.0, 40.0), **user_data) -> list:
    """Initialised (not yet stepped) engine instances of the ensemble
    benchmark. Extra keyword arguments go into every member's user_data."""
    rng = np.random.default_rng(seed)
    sides = np.rint(np.exp(rng.uniform(np.log(side_range[0]), np.log(side_range[1]), n)))
    sims = []
    t_ref = warren_liquidus(c0, Warren1995GB300.DEFAULTS)
    for m, s in enumerate(sides.astype(int)):
        cy, cx = rng.uniform(0.1 * s, 0.9 * s, 2)
        yy, xx = np.mgrid[0:s, 0:s]
        disk = (yy - cy) ** 2 + (xx - cx) ** 2 < 25.0
        if m % 2 == 0:
            ud = dict(user_data, T=float(t_ref - rng.uniform(*dT_range)), seed=int(seed * 1000 + m))
            sim = Warren1995GB300(dimensions=[s, s], dx=4.6e-8, boundary_conditions="NEUMANN",
                                  user_data=ud)
            sim.initialize_fields_and_imported_data()
            phi = np.ones((s, s))
            phi[disk] = 0.0
            sim.fields[0].data[1:-1, 1:-1] = phi
            sim.fields[1].data[1:-1, 1:-1] = c0 + rng.uniform(-1e-3, 1e-3, (s, s))
        else:
            sim = CahnAllenGB300(dimensions=[s, s], dx=1.0, dt=0.1, boundary_conditions="NEUMANN",
                                 user_data=dict(user_data, seed=int(seed * 1000 + m)))
            sim.initialize_fields_and_imported_data()
            sim.fields[0].data[1:-1, 1:-1] = disk.astype(float)
        sims.append(sim)
    return sims


def partition_members(cells, world: int) -> list:
    """Split members (by index) across `world` ranks balancing total cells:
    largest first onto the least-loaded rank (members are independent, so a
    multi-GPU ensemble needs no data-path collective). Returns one sorted
    index list per rank."""
    loads = [0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(cells)), key=lambda i: (-cells[i], i)):
        r = min(range(world), key=lambda r: (loads[r], r))
        parts[r].append(i)
        loads[r] += cells[i]
    return [sorted(p) for p in parts]


class Ensemble:
    """Steps a list of 2-D float32 Warren1995GB300 / CahnAllenGB300 engines
    together. All members must be at the same time step. rows=None picks the
    rows per warp band, the bands per warp and, for four- or eight-row bands,
    persistent or per-step launches with the autotuner. persistent (four- and
    eight-row bands only): each graph chunk of steps is one cooperative launch
    with a grid barrier between steps (default), else one launch per step."""

    def __init__(self, sims, rows: int | None = None, graph_chunk: int = 64, pdl: bool = True,
                 bulk_shortcut: bool = True, use_graph: bool = True, bands: int | None = None,
                 persistent: bool = True):
        if not sims:
            raise ValueError("empty ensemble")
        self.sims = list(sims)
        for s in self.sims:
            if not isinstance(s, (Warren1995GB300, CahnAllenGB300)):
                raise TypeError(f"{type(s).__name__} cannot join an ensemble")
            if len(s.dimensions) != 2:
                raise ValueError("ensemble members are 2-D")
            if s.user_data.get("precision", "fp32") != "fp32":
                raise ValueError("ensemble members are float32")
            if not s._ppf_ready():
                s._begun_simulation = True
                s.just_before_simulating()
        if len({s.time_step_counter for s in self.sims}) != 1 or \
                len({s._ppf_cur for s in self.sims}) != 1:
            raise ValueError("ensemble members must be at the same step")
        self.step = self.sims[0].time_step_counter
        self.cur = self.sims[0]._ppf_cur
        self.graph_chunk = max(2, int(graph_chunk) // 2 * 2)
        self.use_graph = use_graph
        self._pdl = pdl
        self._flags = 0 if bulk_shortcut else L.PPF_TILING_FULL_EVAL
        dev = self.sims[0]._ppf_grid.device
        self.stream = torch.cuda.Stream(dev)
        # the ensemble's own device words live on its stream: freed with the
        # ensemble, their memory is reused only after the stream's work
        with torch.cuda.stream(self.stream):
            self.stepctr = torch.zeros(1, dtype=torch.int64, device=dev)
            # grid-barrier words of the persistent launch (arrivals, generation)
            self.sync = torch.zeros(2, dtype=torch.int32, device=dev)
            self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.status_host = torch.zeros(1, dtype=torch.int32, pin_memory=True)
        self.graphs = {}
        self.persistent = bool(persistent)
        if rows and bands:
            self.rows, self.bands = int(rows), int(bands)
        elif rows:
            self.rows, self.bands = int(rows), 4
        else:
            self.rows, self.bands, self.persistent = self._tune_tiling()
        self.tiling = tiling_struct(1, (self.bands, self.rows), pdl, self._flags)
        self._build()

    @property
    def cells(self) -> int:
        return sum(s._ppf_grid.cells for s in self.sims)

    def _member(self, s, bufs=None) -> L.PpfMember:
        m = L.PpfMember()
        g = s._ppf_grid
        bufs = bufs if bufs is not None else s._ppf_bufs
        m.ny, m.nx = g.kshape
        m.pitch = g.pitch
        m.bc = s._ppf_bc
        m.phi[0] = bufs[0][0].data_ptr()
        m.phi[1] = bufs[1][0].data_ptr()
        if isinstance(s, Warren1995GB300):
            m.model = L.PPF_MODEL_WARREN1995
            m.c[0] = bufs[0][1].data_ptr()
            m.c[1] = bufs[1][1].data_ptr()
            m.seed = int(s.user_data["seed"])
            m.w95 = s._ppf_params()
        else:
            m.model = L.PPF_MODEL_ALLEN_CAHN
            m.ac = s._ppf_params()
        return m

    def _mix_key(self) -> str:
        """The ensemble's member mix (model and grid of every member, sorted)
        as an autotune cache key."""
        import hashlib
        mix = sorted((type(s).__name__, tuple(s._ppf_grid.kshape)) for s in self.sims)
        digest = hashlib.sha1(repr(mix).encode()).hexdigest()[:16]
        from . import autotune
        return autotune.make_key("Ensemble", (len(mix), self.cells), torch.float32, digest)

    def _tune_tiling(self) -> tuple[int, int, bool]:
        """Rows per warp band, bands per warp and persistent launches: each
        candidate times a chunk of steps on scratch copies of every member's
        buffers (the members are untouched)."""
        from . import autotune
        with torch.cuda.stream(self.stream):
            for s in self.sims:
                self.stream.wait_stream(s._ppf_stream)
            scratch = [[[t.clone() for t in bufs] for bufs in s._ppf_bufs] for s in self.sims]
        sync = torch.zeros(2, dtype=torch.int32, device=self.sync.device)
        steps = 8

        def measure(cand):
            tiling = tiling_struct(1, (cand["bands"], cand["rows"]), self._pdl, self._flags)
            members = (L.PpfMember * len(self.sims))(
                *[self._member(s, bufs) for s, bufs in zip(self.sims, scratch)])
            n = len(self.sims)
            nbytes = C.c_size_t()
            L.call("ppf_ensemble_plan_bytes", members, n, C.byref(tiling), C.byref(nbytes))
            table = torch.empty(max(16, nbytes.value), dtype=torch.uint8, device=sync.device)
            plan = L.PpfEnsemblePlan()
            sp = C.c_void_p(self.stream.cuda_stream)
            L.call("ppf_ensemble_build", members, n, C.byref(tiling), ptr(table),
                   C.c_size_t(table.numel()), C.byref(plan), sp)

            barrier = ptr(sync) if cand["persistent"] else None

            def run():
                L.call("ppf_ensemble_run_f32", C.byref(plan), 0, C.c_uint64(0), None, steps,
                       barrier, C.byref(tiling), sp)

            return autotune.time_candidate(run, self.stream, warmup=1, reps=3) / steps

        cands = [{"rows": 2, "bands": b, "persistent": False} for b in (1, 4)] + \
            [{"rows": r, "bands": b, "persistent": p} for r in (4, 8) for b in (1, 4)
             for p in (False, True)]
        best = autotune.pick(self._mix_key(), cands, measure)
        del scratch
        return int(best["rows"]), int(best["bands"]), bool(best["persistent"])

    def _members_key(self) -> bytes:
        """Every member's parameter struct as bytes: the plan (and so every
        captured graph) bakes these in."""
        return b"".join(bytes(self._member(s)) for s in self.sims)

    def _build(self):
        n = len(self.sims)
        self.members = (L.PpfMember * n)(*[self._member(s) for s in self.sims])
        self._key = b"".join(bytes(m) for m in self.members)
        nbytes = C.c_size_t()
        L.call("ppf_ensemble_plan_bytes", self.members, n, C.byref(self.tiling), C.byref(nbytes))
        with torch.cuda.stream(self.stream):
            self.table = torch.empty(max(16, nbytes.value), dtype=torch.uint8,
                                     device=self.stepctr.device)
        self.plan = L.PpfEnsemblePlan()
        for s in self.sims:  # member uploads must land before the first step
            self.stream.wait_stream(s._ppf_stream)
        L.call("ppf_ensemble_build", self.members, n, C.byref(self.tiling), ptr(self.table),
               C.c_size_t(self.table.numel()), C.byref(self.plan), C.c_void_p(self.stream.cuda_stream))

    def _launch(self, parity, step, base, nsteps=1):
        sp = C.c_void_p(self.stream.cuda_stream)
        if nsteps == 1:
            L.call("ppf_ensemble_step_f32", C.byref(self.plan), int(parity), C.c_uint64(step),
                   ptr(base), C.byref(self.tiling), sp)
        else:
            barrier = ptr(self.sync) if self.persistent and self.rows != 2 else None
            L.call("ppf_ensemble_run_f32", C.byref(self.plan), int(parity), C.c_uint64(step),
                   ptr(base), int(nsteps), barrier, C.byref(self.tiling), sp)

    def _watch(self):
        """Status bits of the chunk (a grid-barrier wait that gave up) moved
        into the ensemble's word and copied to the host."""
        sp = C.c_void_p(self.stream.cuda_stream)
        L.call("ppf_status_collect", ptr(self.status), sp)
        with torch.cuda.stream(self.stream):
            self.status_host.copy_(self.status, non_blocking=True)

    def check_status(self, block: bool = True):
        """Raises EngineFault if a launch reported a fault; the barrier words
        are reset so that the ensemble can run again."""
        from .engines.base import EngineFault
        if block:
            self.synchronize()
        bits = int(self.status_host.item())
        if bits:
            self.synchronize()
            bits = int(self.status_host.item())
            with torch.cuda.stream(self.stream):
                self.status.zero_()
                self.sync.zero_()
            self.synchronize()
            self.status_host.zero_()
            raise EngineFault(bits, f"Ensemble of {len(self.sims)} (step {self.step})")

    def _graph(self):
        key = self.cur
        g = self.graphs.get(key)
        if g is not None:
            return g
        sp = C.c_void_p(self.stream.cuda_stream)
        gc_was = gc.isenabled()
        gc.disable()
        exec_ = C.c_void_p()
        L.call("ppf_graph_begin", sp)
        try:
            # one persistent launch for the whole chunk
            self._launch(self.cur, 0, self.stepctr, self.graph_chunk)
            L.call("ppf_counter_add_u64", ptr(self.stepctr), C.c_uint64(self.graph_chunk), sp)
            self._watch()
        finally:
            try:
                L.call("ppf_graph_end", sp, C.byref(exec_))
            finally:
                if gc_was:
                    gc.enable()
        self.graphs[key] = exec_
        return exec_

    def simulate(self, n: int, use_graph: bool | None = None):
        """Advance every member n steps: chunks of graph_chunk steps, each one
        persistent launch (graph-captured unless use_graph is False), and the
        remaining steps in one more launch. A member whose parameters changed
        since the last call (user_data edited) gets a new plan: no captured
        graph replays old constants."""
        n = int(n)
        use_graph = self.use_graph if use_graph is None else use_graph
        sp = C.c_void_p(self.stream.cuda_stream)
        if self._members_key() != self._key:
            self.synchronize()
            for g in self.graphs.values():
                L.call("ppf_graph_destroy", g)
            self.graphs = {}
            self._build()
        self.check_status(block=False)
        if n >= self.graph_chunk:
            g = self._graph() if use_graph else None
            with torch.cuda.stream(self.stream):
                self.stepctr.fill_(self.step)
            while n >= self.graph_chunk:
                if g is not None:
                    L.call("ppf_graph_launch", g, sp)
                else:
                    self._launch(self.cur, self.step, None, self.graph_chunk)
                    self._watch()
                self.step += self.graph_chunk  # even: the parity is unchanged
                n -= self.graph_chunk
        if n > 0:
            self._launch(self.cur, self.step, None, n)
            self._watch()
            self.cur ^= n & 1
            self.step += n
        for s in self.sims:
            s._ppf_cur = self.cur
            s.time_step_counter = self.step
            s._ppf_stream.wait_stream(self.stream)

    def synchronize(self):
        self.stream.synchronize()

    def retrieve_fields_from_GPU(self):
        self.check_status(block=True)
        for s in self.sims:
            s.retrieve_fields_from_GPU()

    def __del__(self):
        try:
            # launches still in flight read the plan table and barrier words
            self.stream.synchronize()
            for g in self.graphs.values():
                L.call("ppf_graph_destroy", g)
        except Exception:
            pass
