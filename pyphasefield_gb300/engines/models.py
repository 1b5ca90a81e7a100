"""The four engines, as drop-in Simulation subclasses.

Each keeps the reference engine's user_data keys and defaults, its field
names and its initial condition, and advances the fields with the CUDA
library instead of numpy:

  DiffusionGB300      <- Engines/Diffusion.py:635-733 (explicit, implicit,
                         Crank-Nicolson, ADI)
  CahnAllenGB300      <- Engines/CahnAllen.py:289-361 (explicit, implicit,
                         Crank-Nicolson, IMEX)
  CahnHilliardGB300   <- Engines/CahnHilliard.py:347-421 (explicit, implicit,
                         Crank-Nicolson, IMEX)
  Warren1995GB300     <- Engines/Warren1995.py:133-207

``make_engines(Base)`` builds the same four classes on any Simulation base
class, e.g. the reference's own pyphasefield.simulation.Simulation.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _lib as L
from ..device import ptr
from ..simulation import Simulation
from .base import GB300Engine

_F = {torch.float32: "f32", torch.float64: "f64"}


_PHASE_SOLVERS = {"implicit": L.PPF_SOLVER_IMPLICIT, "crank-nicolson": L.PPF_SOLVER_CRANK_NICOLSON,
                  "imex": L.PPF_SOLVER_IMEX}


class _ImplicitPhase:
    """user_data["solver"] of the Allen-Cahn and Cahn-Hilliard engines:
    "explicit" (the stencil kernels) or "implicit" / "crank-nicolson" /
    "imex" with "adi" and "gmres", dispatched as CahnAllen.simulation_loop
    (Engines/CahnAllen.py:325-361) and CahnHilliard.simulation_loop
    (Engines/CahnHilliard.py:382-421) do; periodic, as the reference's
    matrices are. user_data["implicit_tol"] bounds the error of the full 2-D
    solve (0: the library default); beyond the Chebyshev bound (16 W M dt >=
    4) that solve is MINRES, capped at user_data["implicit_max_iter"]
    iterations (0: 20000; an unconverged solve raises EngineFault)."""

    PHASE_MODEL = 0

    @property
    def _ppf_phase_solver(self):
        solver = self.user_data.get("solver", "explicit")
        if solver == "explicit":
            return None
        if solver not in _PHASE_SOLVERS:
            raise ValueError(f"{type(self).__name__}: solver must be 'explicit', "
                             f"{', '.join(repr(k) for k in _PHASE_SOLVERS)}; got {solver!r}")
        return _PHASE_SOLVERS[solver]

    def _ppf_phase_prepare(self):
        if self._ppf_phase_solver is None:
            return
        if self.dt is None or self.dx is None:
            raise ValueError(f"{type(self).__name__}: the implicit solvers need dx and dt")
        if min(self.dimensions) < 3:
            raise ValueError("the implicit solvers need >= 3 cells per axis")

    def _ppf_phase_setup(self):
        self._ppf_tmp = self._ppf_scratch = None
        if self._ppf_phase_solver is None:
            return
        g = self._ppf_grid
        self._ppf_tmp = g.empty()
        nbytes = C.c_size_t()
        L.call("ppf_phase_implicit_scratch_bytes", C.byref(g.grid),
               4 if self._ppf_dtype == torch.float32 else 8, C.byref(nbytes))
        self._ppf_scratch = torch.empty(max(16, nbytes.value), dtype=torch.uint8,
                                        device=g.device)

    def _ppf_phase_step(self, src, dst, sp):
        ud = self.user_data
        p = L.PpfImplicitPhaseParams(float(self.dx), float(self.dt), float(ud["M"]),
                                     float(ud["W"]), float(ud["epsilon"]),
                                     float(ud.get("implicit_tol", 0.0)), self.PHASE_MODEL,
                                     self._ppf_phase_solver, 1 if ud.get("adi") else 0,
                                     1 if ud.get("gmres") else 0,
                                     int(ud.get("implicit_max_iter", 0)), 0)
        it = C.c_int32()
        sc = self._ppf_scratch
        L.call(f"ppf_phase_implicit_step_{_F[self._ppf_dtype]}", C.byref(p),
               C.byref(self._ppf_grid.grid), ptr(src[0]), ptr(dst[0]), ptr(self._ppf_tmp),
               ptr(sc), sc.numel(), C.byref(it), sp)
        self._ppf_iterations = it.value

    def _ppf_phase_bc(self):
        if self._ppf_phase_solver is not None and self._boundary_conditions_type is None:
            self._boundary_conditions_type = "PERIODIC"


def _stencil_candidates(sim) -> list:
    """Diffusion / Allen-Cahn launch shapes: temporal depth x tile (2-D),
    tile and planes per CTA along z (3-D)."""
    if len(sim._ppf_grid.kshape) == 2:
        # depth 1: the warp-strip kernel; depth > 1 without a tile or with
        # (0, rows): the marching kernel (segments of `rows`); with a tile:
        # the shared-memory tile kernel
        return [{"temporal_depth": d, "tile": None} for d in (1, 2, 4, 8)] + \
            [{"temporal_depth": d, "tile": (0, 32 * d * f)} for d in (2, 4, 8) for f in (1, 4)] + \
            [{"temporal_depth": d, "tile": t} for d in (1, 2, 4, 8)
             for t in ((128, 32), (64, 32), (256, 16), (128, 16))]
    return [{"tile": (32, 32), "zchunk": z} for z in (8, 12, 16, 24)] + \
        [{"tile": t} for t in ((64, 16), (32, 16), (128, 8))]


_SOLVERS = {"explicit": L.PPF_SOLVER_EXPLICIT, "implicit": L.PPF_SOLVER_IMPLICIT,
            "crank-nicolson": L.PPF_SOLVER_CRANK_NICOLSON}


class _DiffusionMixin(GB300Engine):
    """c += dt*D*lap(c) (engine_ExplicitDiffusion, Engines/Diffusion.py:198-208),
    or one implicit / Crank-Nicolson step (Diffusion.py:210-633) chosen by
    user_data["solver"] ("explicit" | "implicit" | "crank-nicolson") and
    user_data["adi"], as in Diffusion.simulation_loop (:671-720). The
    implicit solvers are periodic on every axis, as the reference's matrices
    are (:18-196); user_data["gmres"] selects the reference's approximate
    GMRES twins, which solve the same systems, so it maps to the same solve.
    user_data["implicit_tol"] bounds the error of the non-ADI 2-D / 3-D
    solves (0: the library default)."""

    NFIELDS = 1

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self.user_data.setdefault("D", 0.1)
        self.user_data.setdefault("solver", "explicit")
        self.user_data.setdefault("gmres", False)
        self.user_data.setdefault("adi", False)
        self.user_data.setdefault("implicit_tol", 0.0)
        self._ppf_defaults()

    def init_fields(self):
        # unit box over the middle half of every axis (Diffusion.py:641-659)
        dim = self.dimensions
        c = np.zeros(dim)
        c[tuple(slice(n // 4, 3 * n // 4) for n in dim)] = 1
        self.add_field(c, "c")

    @property
    def _ppf_solver(self) -> int:
        solver = self.user_data.get("solver", "explicit")
        if solver not in _SOLVERS:
            raise ValueError(f"Diffusion: solver must be one of {sorted(_SOLVERS)}, "
                             f"got {solver!r}")
        return _SOLVERS[solver]

    def _ppf_prepare(self):
        if self.dt is None or self.dx is None:
            raise ValueError("Diffusion needs dx and dt")
        if self._ppf_solver != L.PPF_SOLVER_EXPLICIT and min(self.dimensions) < 3:
            raise ValueError("the implicit solvers need >= 3 cells per axis (the reference's "
                             "periodic matrices are malformed below that)")

    def _ppf_setup(self):
        if self._ppf_solver != L.PPF_SOLVER_EXPLICIT and self._boundary_conditions_type is None:
            # the implicit solvers are periodic; the host ghost cells follow
            self._boundary_conditions_type = "PERIODIC"
        super()._ppf_setup()
        self._ppf_tmp = self._ppf_scratch = None
        if self._ppf_solver != L.PPF_SOLVER_EXPLICIT:
            g = self._ppf_grid
            self._ppf_tmp = g.empty()
            nbytes = C.c_size_t()
            L.call("ppf_implicit_scratch_bytes", C.byref(g.grid),
                   4 if self._ppf_dtype == torch.float32 else 8, C.byref(nbytes))
            self._ppf_scratch = torch.empty(max(16, nbytes.value), dtype=torch.uint8,
                                            device=g.device)

    def _ppf_max_depth(self):
        if self._ppf_solver != L.PPF_SOLVER_EXPLICIT:
            return 1
        return 8 if len(self._ppf_grid.kshape) == 2 else 1

    def _ppf_tune_candidates(self):
        if self._ppf_solver != L.PPF_SOLVER_EXPLICIT:
            return []
        return _stencil_candidates(self)

    def _ppf_params(self):
        return L.PpfDiffusionParams(float(self.dx), float(self.dt), float(self.user_data["D"]))

    def _ppf_implicit_params(self):
        ud = self.user_data
        return L.PpfImplicitDiffusionParams(float(self.dx), float(self.dt), float(ud["D"]),
                                            float(ud.get("implicit_tol", 0.0)), self._ppf_solver,
                                            1 if ud.get("adi", False) else 0)

    def _ppf_step(self, src, dst, depth, step, step_base, sp):
        f = _F[self._ppf_dtype]
        if self._ppf_solver != L.PPF_SOLVER_EXPLICIT:
            p = self._ppf_implicit_params()
            it = C.c_int32()
            sc = self._ppf_scratch
            L.call(f"ppf_diffusion_implicit_step_{f}", C.byref(p), C.byref(self._ppf_grid.grid),
                   ptr(src[0]), ptr(dst[0]), ptr(self._ppf_tmp), ptr(sc), sc.numel(),
                   C.byref(it), sp)
            self._ppf_iterations = it.value
            return
        p = self._ppf_params()
        L.call(f"ppf_diffusion_step_{f}", C.byref(p),
               C.byref(self._ppf_grid.grid), C.byref(self._ppf_bc), ptr(src[0]), ptr(dst[0]),
               C.byref(self._ppf_tiling(depth)), sp)


class _CahnAllenMixin(_ImplicitPhase, GB300Engine):
    """phi += dt*M*(eps^2 lap(phi) - 16 W g'(phi))
    (engine_CahnAllenExplicit, Engines/CahnAllen.py:128-135), or the
    implicit, Crank-Nicolson and IMEX engines (:137-267) by user_data
    "solver" / "adi" / "gmres"."""

    NFIELDS = 1
    PHASE_MODEL = L.PPF_MODEL_ALLEN_CAHN

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        for k, v in dict(M=0.1, epsilon=1.0, W=1.0, solver="explicit", gmres=False,
                         adi=False).items():
            self.user_data.setdefault(k, v)
        self._ppf_defaults()

    def init_fields(self):
        # 0.4995 + 0.001 U[0,1) (CahnAllen.py:311); seeded when user_data has "seed"
        rng = np.random.default_rng(self.user_data["seed"]) if "seed" in self.user_data \
            else np.random
        self.add_field(0.001 * rng.random(self.dimensions) + 0.4995, "phi")

    def _ppf_prepare(self):
        if self.dt is None or self.dx is None:
            raise ValueError("CahnAllen needs dx and dt")
        self._ppf_phase_prepare()

    def _ppf_setup(self):
        self._ppf_phase_bc()
        super()._ppf_setup()
        self._ppf_phase_setup()

    def _ppf_max_depth(self):
        if self._ppf_phase_solver is not None:
            return 1
        return 8 if len(self._ppf_grid.kshape) == 2 else 1

    def _ppf_tune_candidates(self):
        return [] if self._ppf_phase_solver is not None else _stencil_candidates(self)

    def _ppf_params(self):
        ud = self.user_data
        return L.PpfAllenCahnParams(float(self.dx), float(self.dt), float(ud["M"]),
                                    float(ud["epsilon"]), float(ud["W"]))

    def _ppf_step(self, src, dst, depth, step, step_base, sp):
        if self._ppf_phase_solver is not None:
            return self._ppf_phase_step(src, dst, sp)
        p = self._ppf_params()
        L.call(f"ppf_allen_cahn_step_{_F[self._ppf_dtype]}", C.byref(p),
               C.byref(self._ppf_grid.grid), C.byref(self._ppf_bc), ptr(src[0]), ptr(dst[0]),
               C.byref(self._ppf_tiling(depth)), sp)


CH_QUANTUM_F32 = 2.0 ** -24


class _CahnHilliardMixin(_ImplicitPhase, GB300Engine):
    """mu = -eps^2 lap(c) + 4c^3 - 6c^2 + 2c; c += dt*M*lap(mu)
    (engine_CahnHilliardExplicit, Engines/CahnHilliard.py:134-146, with dt;
    dt=None keeps the reference's dt-free update, i.e. dt = 1).

    The device field is u = c - 1/2. In fp32 with conserve_mass (default)
    every face flux is rounded to a multiple of 2^-24 and the initial field
    is rounded to that grid on upload, so the float field's sum is conserved
    exactly. With track_mass (default) the FP64 total mass sum(c) of every
    step is kept in ``mass_history`` (fused into the step kernel).

    user_data "solver" = "implicit" / "crank-nicolson" / "imex" selects the
    reference's other engines (Engines/CahnHilliard.py:148-341); those store
    c itself and track no mass."""

    NFIELDS = 1
    PHASE_MODEL = L.PPF_MODEL_CAHN_HILLIARD

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        for k, v in dict(M=0.1, epsilon=1.0, W=1.0, solver="explicit", gmres=False,
                         adi=False, conserve_mass=True, track_mass=True).items():
            self.user_data.setdefault(k, v)
        self._ppf_defaults()
        self.mass_history: list[float] = []

    def init_fields(self):
        rng = np.random.default_rng(self.user_data["seed"]) if "seed" in self.user_data \
            else np.random
        self.add_field(0.001 * rng.random(self.dimensions) + 0.4995, "phi")

    def _ppf_quantum(self):
        if self._ppf_dtype == torch.float32 and self.user_data.get("conserve_mass", True):
            return CH_QUANTUM_F32
        return 0.0

    def _ppf_prepare(self):
        if self.dx is None:
            raise ValueError("CahnHilliard needs dx")
        self._ppf_phase_prepare()
        self._ch_k = 0
        self._ch_mass_parts = []

    def _ppf_setup(self):
        self._ppf_phase_bc()
        super()._ppf_setup()
        self._ppf_phase_setup()
        chunk = max(2, int(self.user_data.get("graph_chunk", 64)))
        self._ch_mass = torch.zeros(max(chunk, 1024), dtype=torch.float64,
                                    device=self._ppf_grid.device)

    def _ppf_encode(self, j, x):
        if self._ppf_phase_solver is not None:
            return x
        u = np.asarray(x, dtype=np.float64) - 0.5
        q = self._ppf_quantum()
        return np.rint(u / q) * q if q else u

    def _ppf_decode(self, j, x):
        return x if self._ppf_phase_solver is not None else x + 0.5

    def _ppf_max_depth(self):
        return 1

    def _ppf_params(self):
        ud = self.user_data
        dt = 1.0 if self.dt is None else float(self.dt)
        p = L.PpfCahnHilliardParams(float(self.dx), dt, float(ud["M"]), float(ud["epsilon"]),
                                    self._ppf_quantum())
        p.centered = 1
        p.reserved = 0
        return p

    def _ppf_tracks_mass(self):
        return self._ppf_phase_solver is None and self.user_data.get("track_mass", True)

    def _ppf_segment_begin(self, nsteps, stream):
        self._ch_k = 0
        if self._ppf_tracks_mass():
            if nsteps > self._ch_mass.numel():
                self._ch_mass = torch.zeros(nsteps, dtype=torch.float64,
                                            device=self._ppf_grid.device)
            self._ch_mass[:nsteps].zero_()

    def _ppf_segment_end(self, nsteps, stream):
        if self._ppf_tracks_mass():
            with torch.cuda.stream(stream):
                self._ch_mass_parts.append(self._ch_mass[:nsteps].clone())

    def _ppf_step(self, src, dst, depth, step, step_base, sp):
        if self._ppf_phase_solver is not None:
            return self._ppf_phase_step(src, dst, sp)
        p = self._ppf_params()
        mass = None
        if self.user_data.get("track_mass", True):
            mass = self._ch_mass[self._ch_k]
        self._ch_k += 1
        L.call(f"ppf_cahn_hilliard_step_{_F[self._ppf_dtype]}", C.byref(p),
               C.byref(self._ppf_grid.grid), C.byref(self._ppf_bc), ptr(src[0]), ptr(dst[0]),
               ptr(mass), ptr(self._ppf_status), C.byref(self._ppf_tiling(depth)), sp)

    def collect_mass_history(self) -> np.ndarray:
        """FP64 total mass sum(c) after every step run so far (host sync)."""
        if self._ch_mass_parts:
            self.synchronize()
            half = 0.5 * self._ppf_grid.cells
            new = torch.cat(self._ch_mass_parts).cpu().numpy() + half
            self.mass_history.extend(new.tolist())
            self._ch_mass_parts = []
        return np.asarray(self.mass_history)

    def status_flags(self) -> int:
        """The engine's sticky status word (PPF_STATUS_* bits seen so far
        and not yet raised as EngineFault; host sync)."""
        self.synchronize()
        return int(self._ppf_status.item())


class _Warren1995Mixin(GB300Engine):
    """Binary Ni-Cu isothermal solidification (Engines/Warren1995.py:50-207)."""

    NFIELDS = 2
    DEFAULTS = dict(T_mA=1728.0, T_mB=1358.0, L_A=2350000000.0, L_B=1728000000.0, s_A=0.37,
                    s_B=0.29, D_L=1e-9, D_S=1e-13, B_A=0.0033, B_B=0.0039, v_m=0.00000742,
                    R=8.314, y_e=0.04, T=1574.0, alpha=0.3, diamond_size=15)

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        for k, v in self.DEFAULTS.items():
            self.user_data.setdefault(k, v)
        self.user_data.setdefault("seed", 0)
        self._ppf_defaults()

    def init_fields(self):
        # phi = 1 (liquid) with a diamond of phi = 0 (solid) at the centre,
        # c = 0.40831 (Warren1995.py:172-185)
        dim = self.dimensions
        phi = np.ones(dim)
        ds = int(self.user_data["diamond_size"])
        for i in range(ds):
            phi[int(dim[0] / 2 - i):int(dim[0] / 2 + i),
                int(dim[1] / 2 - (ds - i)):int(dim[1] / 2 + (ds - i))] = 0
        self.add_field(phi, "phi")
        self.add_field(np.full(dim, 0.40831), "c")

    def _ppf_prepare(self):
        # Warren1995.just_before_simulating (:193-203)
        ud = self.user_data
        if self.dx is None:
            raise ValueError("Warren1995 needs dx (cell spacing in m)")
        if len(self.dimensions) != 2:
            raise ValueError("Warren1995 is a 2-D model")
        dx = float(self.dx)
        self.set_time_step_length(dx ** 2 / 5.0 / ud["D_L"])
        ud["d"] = dx / 0.94
        r2 = np.sqrt(2)
        ud["ebar"] = np.sqrt(6 * r2 * ud["s_A"] * ud["d"] / ud["T_mA"])
        ud["W_A"] = 3 * ud["s_A"] / (r2 * ud["T_mA"] * ud["d"])
        ud["W_B"] = 3 * ud["s_B"] / (r2 * ud["T_mB"] * ud["d"])
        ud["M_A"] = (ud["T_mA"] ** 2) * ud["B_A"] / (6 * r2 * ud["L_A"] * ud["d"])
        ud["M_B"] = (ud["T_mB"] ** 2) * ud["B_B"] / (6 * r2 * ud["L_B"] * ud["d"])

    def _ppf_tune_candidates(self):
        return [{"tile": (0, rows)} for rows in (2, 4, 8)]

    def _ppf_tiling(self, depth: int):
        t = super()._ppf_tiling(depth)
        if self.user_data.get("tile") is None and self._ppf_dtype == torch.float32:
            # rows per warp when neither the user nor the autotuner chose:
            # eight from 2^22 cells up, where each warp then keeps more loads
            # in flight and the grid still fills several waves of CTAs
            # (per step: 2048^2 22.5 -> 21.0 us, 3072^2 45.7 -> 36.9 us,
            # 4096^2 77.4 -> 55.3 us, every cell on the full update 122 -> 96
            # us), two below (1024^2: 10.9 us against 12.9 with four rows:
            # about one wave of the larger bands)
            t.tile_y = 8 if self._ppf_grid.cells >= 1 << 22 else 2
        return t

    def _ppf_params(self):
        ud = self.user_data
        vals = dict(ud, dx=float(self.dx), dt=float(self.dt))
        return L.PpfWarren1995Params(*[float(vals[n]) for n in L.WARREN_PARAM_NAMES])

    def _ppf_step(self, src, dst, depth, step, step_base, sp):
        p = self._ppf_params()
        L.call(f"ppf_warren1995_step_{_F[self._ppf_dtype]}", C.byref(p),
               C.byref(self._ppf_grid.grid), C.byref(self._ppf_bc), ptr(src[0]), ptr(src[1]),
               ptr(dst[0]), ptr(dst[1]), C.c_uint64(int(self.user_data["seed"])),
               C.c_uint64(int(step)), ptr(step_base), C.byref(self._ppf_tiling(depth)), sp)


def make_engines(base=Simulation) -> dict:
    """Build the engine classes on `base` (any class with the reference
    Simulation interface): Diffusion, CahnAllen (= AllenCahn), CahnHilliard,
    Warren1995, NCGPU and NCGPU_new. Returns {name: class}."""
    from .ncgpu import make_ncgpu, make_ncgpu_new
    out = {}
    for name, mix in (("DiffusionGB300", _DiffusionMixin), ("CahnAllenGB300", _CahnAllenMixin),
                      ("CahnHilliardGB300", _CahnHilliardMixin),
                      ("Warren1995GB300", _Warren1995Mixin)):
        out[name] = type(name, (mix, base), {"__module__": __name__,
                                            "__doc__": mix.__doc__})
    out["AllenCahnGB300"] = out["CahnAllenGB300"]
    out["NCGPUGB300"] = make_ncgpu(base)
    out["NCGPU_newGB300"] = make_ncgpu_new(base)
    return out


_engines = make_engines(Simulation)
DiffusionGB300 = _engines["DiffusionGB300"]
CahnAllenGB300 = _engines["CahnAllenGB300"]
AllenCahnGB300 = CahnAllenGB300
CahnHilliardGB300 = _engines["CahnHilliardGB300"]
Warren1995GB300 = _engines["Warren1995GB300"]
