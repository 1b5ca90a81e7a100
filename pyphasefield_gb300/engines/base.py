"""GB300Engine: the device half of every engine in this package.

Mixed into a Simulation subclass (this package's, or the reference's own
pyphasefield.simulation.Simulation through make_engines), it replaces the
reference's per-step loop (Simulation.simulate, simulation.py:245-271) and
its numba device utilities (ppf_gpu_utils.send_fields_to_GPU /
retrieve_fields_from_GPU / apply_boundary_conditions, ppf_gpu_utils.py:
396-514):

* fields live on the device as float32 (default) or float64, interior only,
  in two ping-pong buffer sets; the boundary rule is fused into every
  kernel's tile load, so apply_boundary_conditions is a no-op on device;
* simulate(n) advances n steps in captured CUDA graphs of `graph_chunk`
  launches (each launch with programmatic dependent launch), split at
  autosave boundaries so autosave cadence and time_step_counter behave as in
  the reference;
* send_fields_to_GPU / retrieve_fields_from_GPU move the interiors between
  Field.data (float64, ghosts refilled on the host) and the device.

User-data keys added to the reference's: precision ("fp32" | "fp64"),
temporal_depth (steps per HBM pass, 2-D Diffusion/Allen-Cahn), tile
((tile_x, tile_y) or None; Warren1995: (0, rows per warp band), chosen by
grid size when None), zchunk (planes per CTA, 3-D), autotune (bool: time the
launch shapes on scratch copies and cache the fastest), bulk_shortcut
(bool, Warren1995), pdl (bool), use_graph (bool), graph_chunk (int),
check_status (bool, default True).

Failure detection: after every chunk of steps (inside the captured graph)
the engine runs the NaN/Inf sentinel over its fields (ppf_check_finite_*),
moves the library's status bits (a bounded barrier wait that gave up, a
Cahn-Hilliard range overflow) into its own sticky status word
(ppf_status_collect) and copies that word to pinned host memory. The host
reads the copy at the next chunk boundary (waiting for the chunk before the
last, so the device stays a chunk ahead), at every autosave and in
retrieve_fields_from_GPU, and raises EngineFault on any set bit: a run never
carries on from a state a kernel reported as corrupt. The library's word is
shared by every engine on a device; whichever engine collects it first
reports the fault.
"""
from __future__ import annotations

import collections
import contextlib
import ctypes as C
import gc
import hashlib
import inspect
from pathlib import Path

import numpy as np
import torch

from .. import _lib as L
from ..device import DeviceGrid, boundary_struct, ptr, require_cuda, tiling_struct
from ..simulation import fill_ghosts_host

COMMON_DEFAULTS = dict(precision="fp32", temporal_depth=1, tile=None, pdl=True,
                       use_graph=True, graph_chunk=64, check_status=True)

#: captured graphs kept per engine (one per distinct parameter set)
MAX_GRAPHS = 8

_STATUS_NAMES = ((L.PPF_STATUS_TIMEOUT, "a bounded barrier wait timed out (tile not written)"),
                 (L.PPF_STATUS_NONFINITE, "a field holds NaN or Inf"),
                 (L.PPF_STATUS_RANGE, "a value left the kernel's representable range"),
                 (L.PPF_STATUS_NOT_CONVERGED, "an iterative solve did not converge"))


try:
    from torch.cuda import nvtx as _nvtx
except Exception:  # pragma: no cover - torch without NVTX
    _nvtx = None


@contextlib.contextmanager
def nvtx_range(name: str):
    """NVTX range on the host timeline (shown by Nsight Systems / ncu
    --nvtx): simulate calls, graph replays, eager passes, transfers."""
    if _nvtx is None:
        yield
        return
    _nvtx.range_push(name)
    try:
        yield
    finally:
        _nvtx.range_pop()


def _save_npz(sim, step: int) -> None:
    """The reference's checkpoint format: np.savez of every field's interior
    keyed by field name, to <save_path>/step_<step>.npz."""
    if not sim._save_path:
        print("self._save_path not defined, aborting save!")
        return
    loc = Path(sim._save_path)
    loc.mkdir(parents=True, exist_ok=True)
    np.savez(str(loc) + "/step_" + str(int(step)), **{f.name: f.get_cells() for f in sim.fields})


class EngineFault(RuntimeError):
    """A kernel reported a fault through the device status word."""

    def __init__(self, bits: int, where: str):
        self.bits = bits
        names = [n for b, n in _STATUS_NAMES if bits & b] or [f"status bits {bits:#x}"]
        super().__init__(f"{where}: " + "; ".join(names))


class GB300Engine:
    #: number of fields the engine advances together
    NFIELDS = 1

    # ------------------------------------------------------------ subclass API
    def _ppf_params(self):
        """Return the ctypes params struct for the library call."""
        raise NotImplementedError

    def _ppf_step(self, src, dst, depth: int, step: int, step_base, stream_ptr):
        """Launch one pass advancing `depth` steps from buffers src to dst."""
        raise NotImplementedError

    def _ppf_max_depth(self) -> int:
        return 1

    def _ppf_encode(self, j: int, x: np.ndarray) -> np.ndarray:
        """Host value -> stored value of field j (identity by default)."""
        return x

    def _ppf_decode(self, j: int, x: np.ndarray) -> np.ndarray:
        return x

    def _ppf_prepare(self):
        """Engine-specific set-up before the device copy (derived params)."""

    def _ppf_segment_begin(self, nsteps: int, stream):
        """Launches issued before a run of steps (captured in graphs)."""

    def _ppf_segment_end(self, nsteps: int, stream):
        """Host bookkeeping after a run of steps (not captured)."""

    # ------------------------------------------------------------ helpers
    def _ppf_defaults(self):
        for k, v in COMMON_DEFAULTS.items():
            self.user_data.setdefault(k, v)

    @property
    def _ppf_dtype(self):
        p = self.user_data.get("precision", "fp32")
        if p not in ("fp32", "fp64"):
            raise ValueError(f"precision must be 'fp32' or 'fp64', got {p!r}")
        return torch.float32 if p == "fp32" else torch.float64

    def _ppf_ready(self) -> bool:
        return getattr(self, "_ppf_bufs", None) is not None

    def _ppf_setup(self):
        dev = require_cuda()
        if not self.fields or len(self.fields) != self.NFIELDS:
            raise RuntimeError(f"{type(self).__name__} needs {self.NFIELDS} field(s); "
                               "call initialize_fields_and_imported_data() first")
        shape = self.fields[0].get_cells().shape
        self._ppf_release_graphs()
        self._ppf_grid = DeviceGrid(shape, self._ppf_dtype, dev)
        self._ppf_bufs = [[self._ppf_grid.empty() for _ in range(self.NFIELDS)] for _ in range(2)]
        self._ppf_cur = 0
        self._ppf_stream = torch.cuda.Stream(dev)
        self._ppf_bc = boundary_struct(self, self._ppf_grid, self.NFIELDS)
        self._ppf_stepctr = torch.zeros(1, dtype=torch.int64, device=dev)
        # the buffers' zero fills ran on the current stream
        self._ppf_stream.wait_stream(torch.cuda.current_stream(dev))
        self._ppf_graphs = collections.OrderedDict()
        self._ppf_staging = []
        self._ppf_status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._ppf_status_host = torch.zeros(1, dtype=torch.int32, pin_memory=True)
        self._ppf_status_events = collections.deque()
        self._uses_gpu = True

    def _ppf_release_graphs(self):
        for g in getattr(self, "_ppf_graphs", {}).values():
            L.call("ppf_graph_destroy", g)
        self._ppf_graphs = collections.OrderedDict()

    # ------------------------------------------------------------ status
    def _ppf_watch(self, stream):
        """Launches issued after a chunk of steps (captured with it): the
        NaN/Inf sentinel on the current fields, the library status bits
        moved into the engine's word, and the word copied to pinned host
        memory."""
        if not self.user_data.get("check_status", True):
            return
        sp = C.c_void_p(stream.cuda_stream)
        f = "f32" if self._ppf_dtype == torch.float32 else "f64"
        st = ptr(self._ppf_status)
        for t in self._ppf_bufs[self._ppf_cur]:
            L.call(f"ppf_check_finite_{f}", ptr(t), C.byref(self._ppf_grid.grid), st, sp)
        L.call("ppf_status_collect", st, sp)
        with torch.cuda.stream(stream):
            self._ppf_status_host.copy_(self._ppf_status, non_blocking=True)

    def _ppf_watch_launches(self) -> int:
        """Kernels _ppf_watch launches (the copy is not a kernel)."""
        return self.NFIELDS + 1 if self.user_data.get("check_status", True) else 0

    def _ppf_mark(self):
        """Records the point after a chunk's status copy (host side)."""
        if self.user_data.get("check_status", True):
            ev = torch.cuda.Event()
            ev.record(self._ppf_stream)
            self._ppf_status_events.append(ev)

    def _ppf_check_status(self, block: bool, where: str = "simulate"):
        """Raises EngineFault if a chunk reported a fault. block=False waits
        only for chunks two or more behind the newest, so the device keeps
        one chunk queued; block=True waits for everything issued."""
        if not self._ppf_ready():
            return
        evs = self._ppf_status_events
        if block:
            if evs:
                evs[-1].synchronize()
                evs.clear()
        else:
            while len(evs) > 1:
                evs.popleft().synchronize()
        bits = int(self._ppf_status_host.item())
        if bits:
            self.synchronize()
            bits = int(self._ppf_status_host.item())
            with torch.cuda.stream(self._ppf_stream):
                self._ppf_status.zero_()
            self._ppf_stream.synchronize()
            self._ppf_status_host.zero_()
            raise EngineFault(bits, f"{type(self).__name__} {where} (step "
                                    f"{self.time_step_counter})")

    def __del__(self):
        try:
            if getattr(self, "_ppf_stream", None) is not None:
                # work in flight still reads the buffers freed with the engine
                self._ppf_stream.synchronize()
            self._ppf_checkpoint_wait()
            ck = getattr(self, "_ppf_ckpt", None)
            if ck is not None:
                ck["pool"].shutdown(wait=True)
            self._ppf_release_graphs()
        except Exception:
            pass

    def _ppf_tune_candidates(self) -> list:
        """Launch shapes the autotuner may try (user_data updates)."""
        return []

    def _ppf_autotune(self):
        """Pick tile / temporal depth by timing candidates on scratch copies
        of the current fields (user_data["autotune"] = True); the choice is
        cached per kernel, shape, dtype and device (autotune.py)."""
        from .. import autotune

        cands = self._ppf_tune_candidates()
        if len(cands) < 2:
            return
        key = autotune.make_key(type(self).__name__, self._ppf_grid.kshape, self._ppf_dtype,
                                str(len(self.dimensions)))
        s = self._ppf_stream
        sp = C.c_void_p(s.cuda_stream)
        with torch.cuda.stream(s):
            scratch = [[t.clone() for t in self._ppf_bufs[self._ppf_cur]] for _ in range(2)]
        saved = {k: self.user_data.get(k) for c in cands for k in c}

        def measure(cand):
            self.user_data.update(cand)
            depth = max(1, min(int(self.user_data.get("temporal_depth", 1)), self._ppf_max_depth()))
            flip = [0]

            def run():
                self._ppf_step(scratch[flip[0]], scratch[1 - flip[0]], depth, 0, None, sp)
                flip[0] ^= 1

            return autotune.time_candidate(run, s) / depth

        try:
            best = autotune.pick(key, cands, measure)
        finally:
            self.user_data.update(saved)
        self.user_data.update(best)
        self._ppf_graphs_reset()

    def _ppf_graphs_reset(self):
        self._ppf_release_graphs()

    def _ppf_tiling(self, depth: int):
        ud = self.user_data
        flags = 0 if ud.get("bulk_shortcut", True) else L.PPF_TILING_FULL_EVAL
        return tiling_struct(depth, ud.get("tile"), ud.get("pdl", True), flags, ud.get("zchunk", 0))

    # ------------------------------------------------------------ lifecycle
    def just_before_simulating(self):
        t = self._temperature_type
        if t not in (None, "ISOTHERMAL", "LINEAR_GRADIENT"):
            raise NotImplementedError(f"temperature type {t!r} is not supported (XDMF input "
                                      "needs meshio)")
        self._ppf_prepare()
        self._ppf_setup()
        fill_ghosts_host(self)
        self.send_fields_to_GPU()
        if self.user_data.get("autotune", False):
            self._ppf_autotune()

    def send_fields_to_GPU(self):
        if not self._ppf_ready():
            self._ppf_setup()
        s = self._ppf_stream
        with nvtx_range("ppf.send_fields_to_GPU"):
            self._ppf_send(s)

    def _ppf_send(self, s):
        self._ppf_staging = [
            self._ppf_grid.upload(self._ppf_bufs[self._ppf_cur][j],
                                  self._ppf_encode(j, f.get_cells()), s)
            for j, f in enumerate(self.fields)]

    def retrieve_fields_from_GPU(self):
        if not self._ppf_ready():
            return
        self._ppf_check_status(True, "retrieve_fields_from_GPU")
        s = self._ppf_stream
        with nvtx_range("ppf.retrieve_fields_from_GPU"):
            for j, f in enumerate(self.fields):
                f.data[f._slice] = self._ppf_decode(
                    j, self._ppf_grid.download(self._ppf_bufs[self._ppf_cur][j], s))
        self._ppf_staging = []
        fill_ghosts_host(self)

    def apply_boundary_conditions(self):
        if self._ppf_ready():
            return  # fused into every kernel's tile load
        fill_ghosts_host(self)

    def update_temperature_field(self, force_cpu=False):
        """One step of the temperature law (simulation.py:303-333). None of the
        four engines reads the temperature field (Warren1995 takes the scalar
        T of user_data), so it stays a host field that advances with the
        step count."""
        self._ppf_advance_temperature(1)

    def _ppf_advance_temperature(self, nsteps: int):
        t = self._temperature_type
        if t == "LINEAR_GRADIENT" and self.temperature is not None and self._dTdt:
            # closed form of nsteps per-step increments dTdt * dt
            self.temperature.data += nsteps * self._dTdt * self.dt
        elif t not in (None, "ISOTHERMAL", "LINEAR_GRADIENT"):
            raise NotImplementedError(f"temperature type {t!r} is not supported")

    def simulation_loop(self):
        """Advance one step on the device (the reference's engine call)."""
        if not self._ppf_ready():
            self.just_before_simulating()
        self._ppf_advance(1, self.time_step_counter)

    def simulate(self, number_of_timesteps):
        with nvtx_range(f"ppf.simulate {type(self).__name__} n={int(number_of_timesteps)}"):
            self._ppf_simulate(number_of_timesteps)

    def _ppf_simulate(self, number_of_timesteps):
        if not self._begun_simulation or not self._ppf_ready():
            self._begun_simulation = True
            self.just_before_simulating()
        n = int(number_of_timesteps)
        rate = self._autosave_rate if self._autosave_flag else None
        while n > 0:
            chunk = n
            if rate:
                chunk = min(chunk, rate - self.time_step_counter % rate)
            # the reference increments the counter before each engine call;
            # the step index keyed into the noise is the counter before it
            try:
                self._ppf_advance(chunk, self.time_step_counter)
            except EngineFault:
                # the counter covers the steps launched before the fault
                self.time_step_counter += self._ppf_done
                raise
            self.time_step_counter += chunk
            self._ppf_advance_temperature(chunk)
            n -= chunk
            if rate and self.time_step_counter % rate == 0:
                self._ppf_check_status(True, "autosave")
                self._ppf_checkpoint()
        self._ppf_checkpoint_wait()

    # ------------------------------------------------------------ autosave
    def _ppf_checkpoint(self):
        """Autosave without stopping the device (simulation.py:267-271 saves
        synchronously): the state is copied on the device into one of two
        snapshot slots, then to pinned host memory on a copy stream, and a
        writer thread fills Field.data and writes step_<counter>.npz while
        the next steps run. simulate() returns after every write finished,
        with Field.data holding the last autosaved state, as in the
        reference."""
        with nvtx_range(f"ppf.autosave step {self.time_step_counter}"):
            self._ppf_checkpoint_issue()

    def _ppf_checkpoint_issue(self):
        import concurrent.futures as cf
        ck = getattr(self, "_ppf_ckpt", None)
        g = self._ppf_grid
        if ck is None:
            ck = self._ppf_ckpt = {
                "pool": cf.ThreadPoolExecutor(max_workers=1), "stream": torch.cuda.Stream(g.device),
                "slots": [{"dev": [g.empty() for _ in range(self.NFIELDS)],
                           "host": [torch.empty(g.alloc_shape, dtype=g.dtype, pin_memory=True)
                                    for _ in range(self.NFIELDS)], "job": None}
                          for _ in range(2)], "next": 0}
        slot = ck["slots"][ck["next"]]
        ck["next"] ^= 1
        if slot["job"] is not None:
            slot["job"].result()  # the slot's previous write is done with its buffers
        s, cs = self._ppf_stream, ck["stream"]
        with torch.cuda.stream(s):
            for j in range(self.NFIELDS):
                slot["dev"][j].copy_(self._ppf_bufs[self._ppf_cur][j])
        taken = torch.cuda.Event()
        taken.record(s)
        cs.wait_event(taken)
        with torch.cuda.stream(cs):
            for j in range(self.NFIELDS):
                slot["host"][j].copy_(slot["dev"][j], non_blocking=True)
        done = torch.cuda.Event()
        done.record(cs)
        slot["job"] = ck["pool"].submit(self._ppf_write_checkpoint, slot, done,
                                        self.time_step_counter)

    def _ppf_write_checkpoint(self, slot, done, step):
        done.synchronize()
        g = self._ppf_grid
        for j, f in enumerate(self.fields):
            host = slot["host"][j][..., : g.kshape[-1]].numpy().astype(np.float64)
            f.data[f._slice] = self._ppf_decode(j, host.reshape(g.user_shape))
        fill_ghosts_host(self)
        if "step" in inspect.signature(self.save_simulation).parameters:
            self.save_simulation(step=step)
        else:
            # the reference's save_simulation (simulation.py:399-420) names the
            # file by the live counter, which has moved on by now: write the
            # same file under the step that was snapshotted
            _save_npz(self, step)

    def _ppf_checkpoint_wait(self):
        ck = getattr(self, "_ppf_ckpt", None)
        if ck is not None:
            for slot in ck["slots"]:
                if slot["job"] is not None:
                    slot["job"].result()
                    slot["job"] = None

    # ------------------------------------------------------------ stepping
    def _ppf_passes(self, nsteps: int) -> list[int]:
        k = max(1, min(int(self.user_data.get("temporal_depth", 1)), self._ppf_max_depth()))
        passes = [k] * (nsteps // k)
        if nsteps % k:
            passes.append(nsteps % k)
        return passes

    def _ppf_launch_pass(self, depth, step, step_base):
        src = self._ppf_bufs[self._ppf_cur]
        dst = self._ppf_bufs[1 - self._ppf_cur]
        self._ppf_step(src, dst, depth, step, step_base, C.c_void_p(self._ppf_stream.cuda_stream))
        self._ppf_cur ^= 1

    def _ppf_state_key(self):
        """What a captured graph bakes in besides the buffers: every
        user_data value (parameters, tiling, seed, ...), dt, dx and the
        boundary struct. A graph is reused only while all of it is unchanged,
        so editing user_data between simulate() calls never replays stale
        constants."""
        items = []
        for k, v in sorted(self.user_data.items(), key=lambda kv: str(kv[0])):
            if isinstance(v, np.ndarray):
                v = (v.shape, v.dtype.str,
                     hashlib.sha1(np.ascontiguousarray(v).tobytes()).hexdigest())
            elif isinstance(v, torch.Tensor):
                v = ("tensor", v.data_ptr(), tuple(v.shape), v._version)
            else:
                v = repr(v)
            items.append((str(k), v))
        return (tuple(items), repr(self.dt), repr(self.dx), bytes(self._ppf_bc))

    def _ppf_graph(self, depths: tuple[int, ...]):
        key = (self._ppf_cur, depths, self._ppf_state_key())
        g = self._ppf_graphs.get(key)
        if g is not None:
            self._ppf_graphs.move_to_end(key)
            return g
        while len(self._ppf_graphs) >= MAX_GRAPHS:
            L.call("ppf_graph_destroy", self._ppf_graphs.popitem(last=False)[1])
        s = self._ppf_stream
        sp = C.c_void_p(s.cuda_stream)
        cur0 = self._ppf_cur
        total = sum(depths)
        # No Python garbage collection while capturing: collecting another
        # engine would free its pinned staging buffers and graphs, and those
        # CUDA calls would invalidate the capture.
        gc_was_enabled = gc.isenabled()
        gc.disable()
        L.call("ppf_graph_begin", sp)
        exec_ = C.c_void_p()
        try:
            with torch.cuda.stream(s):
                self._ppf_segment_begin(total, s)
                off = 0
                for d in depths:
                    self._ppf_launch_pass(d, off, self._ppf_stepctr)
                    off += d
                L.call("ppf_counter_add_u64", ptr(self._ppf_stepctr), C.c_uint64(total), sp)
                self._ppf_watch(s)
        finally:
            try:
                L.call("ppf_graph_end", sp, C.byref(exec_))
            finally:
                self._ppf_cur = cur0
                if gc_was_enabled:
                    gc.enable()
        self._ppf_graphs[key] = exec_
        return exec_

    def _ppf_advance(self, nsteps: int, step0: int):
        """Advance nsteps from absolute step index step0 (noise key)."""
        if nsteps <= 0:
            return
        self._ppf_done = 0
        passes = self._ppf_passes(nsteps)
        ud = self.user_data
        chunk = max(2, int(ud.get("graph_chunk", 64)) // 2 * 2)
        s = self._ppf_stream
        sp = C.c_void_p(s.cuda_stream)
        i = 0
        step = step0
        if ud.get("use_graph", True) and len(passes) >= chunk:
            depths = tuple(passes[:chunk])
            if all(d == depths[0] for d in depths):
                g = self._ppf_graph(depths)
                span = sum(depths)
                with torch.cuda.stream(s):
                    self._ppf_stepctr.fill_(step)
                while len(passes) - i >= chunk:
                    self._ppf_check_status(False)
                    with nvtx_range(f"ppf.graph {span} steps from {step}"):
                        L.call("ppf_graph_launch", g, sp)
                    self._ppf_mark()
                    self._ppf_segment_end(span, s)
                    i += chunk
                    step += span
                    self._ppf_done += span
        if i < len(passes):
            self._ppf_check_status(False)
            rest = passes[i:]
            with torch.cuda.stream(s), nvtx_range(f"ppf.eager {sum(rest)} steps from {step}"):
                self._ppf_segment_begin(sum(rest), s)
                for d in rest:
                    self._ppf_launch_pass(d, step, None)
                    step += d
                self._ppf_watch(s)
            self._ppf_mark()
            self._ppf_segment_end(sum(rest), s)

    # ------------------------------------------------------------ access
    def device_fields(self) -> list[torch.Tensor]:
        """Views of the current device fields (interior only, stored values)."""
        return [self._ppf_grid.view(t) for t in self._ppf_bufs[self._ppf_cur]]

    def synchronize(self):
        if self._ppf_ready():
            self._ppf_stream.synchronize()
