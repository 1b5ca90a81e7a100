"""NCGPUGB300: the reference's NCGPU engine (Engines/NCGPU.py:329-532) on the
CUDA library: alloy solidification (2 to 6 components) with a phase field,
two quaternion orientation fields and the fractions of all but the last
component, thermodynamics from a TDB file (read by pyphasefield_gb300.tdb
instead of pycalphad: pure-element energies, ideal mixing and binary
Redlich-Kister excess terms).

Fields, in the reference's order: phi (1 = solid), q1, q4, c_<component> for
every component but the last (sorted). user_data keys as the reference: d_ratio (4), sim_type ("seed"
places one seed at the centre; anything else leaves the melt), melt_angle,
seed_angle, initial_concentration_array; added: seed (noise stream),
noise_scale (1 = the reference's Langevin term on dF/dc, 0 = none).
dt is the reference's dx^2 / 5 / D_L / 8. precision defaults to "fp64"
(float32 runs; its threshold branches part from float64 within a few
steps). Periodic or zero-gradient
boundaries; the temperature field is ISOTHERMAL or a LINEAR_GRADIENT, with
or without dTdt: the device copy rises by dTdt * dt after every step, as
the reference's update_thermal_gradient kernels do (ppf_gpu_utils.py:
326-334); with dTdt the pure-element energies are evaluated at every step
instead of once per run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _lib as L
from ..device import ptr
from ..simulation import Simulation
from ..tdb import Database
from .base import GB300Engine

_F = {torch.float32: "f32", torch.float64: "f64"}


def ncgpu_parameters(db: Database, dx: float, d_ratio: float = 4.0) -> dict:
    """NCGPU.init_tdb_params (NCGPU.py:336-373): per-component latent heat,
    melting point, surface energy and kinetic coefficient from the TDB's
    <COMP>_L / _TM / _S / _B functions, the derived W and M, and the scalar
    functions D_S, D_L, V_M, M_Q, H, Y_E."""
    comps = db.elements
    if not 2 <= len(comps) <= L.PPF_NCGPU_MAX_COMP:
        raise NotImplementedError(f"NCGPU: 2 to {L.PPF_NCGPU_MAX_COMP} components "
                                  f"(the TDB lists {comps})")
    d = dx * d_ratio
    ud = {"d": d, "R": 8.314}
    for key, fn in (("L", "_L"), ("T_M", "_TM"), ("S", "_S"), ("B", "_B")):
        ud[key] = [db.scalar(c + fn) for c in comps]
    ud["W"] = [3 * s / (np.sqrt(2) * tm * d) for s, tm in zip(ud["S"], ud["T_M"])]
    # the reference divides the mobility by a fixed 1574 (NCGPU.py:362)
    ud["M"] = [tm ** 2 * b / (6 * np.sqrt(2) * lat * d) / 1574.0
               for tm, b, lat in zip(ud["T_M"], ud["B"], ud["L"])]
    for key, fn in (("D_S", "D_S"), ("D_L", "D_L"), ("v_m", "V_M"), ("M_qmax", "M_Q"),
                    ("H", "H"), ("y_e", "Y_E")):
        ud[key] = db.scalar(fn)
    ud["ebar"] = float(np.sqrt(6 * np.sqrt(2) * ud["S"][1] * d / ud["T_M"][1]))
    ud["eqbar"] = 0.5 * ud["ebar"]
    ud["beta"] = 1.5
    ud["dt"] = dx ** 2 / 5.0 / ud["D_L"] / 8
    return ud


def gibbs_table(db: Database):
    """(gibbs[2][MAX_COMP][4][10], npieces[2][MAX_COMP]) for PpfNcgpuParams:
    phase 0 the solid (first phase in sorted order), 1 the liquid; components
    sorted."""
    if len(db.phases) != 2:
        raise NotImplementedError(f"NCGPU: two phases expected (the TDB lists {db.phases})")
    table = np.zeros((2, L.PPF_NCGPU_MAX_COMP, 4, 10))
    npieces = np.zeros((2, L.PPF_NCGPU_MAX_COMP), dtype=np.int32)
    for ph, phase in enumerate(db.phases):
        for cp, comp in enumerate(db.elements):
            pieces = db.params.get((phase, comp))
            if pieces is None:
                raise ValueError(f"TDB has no G({phase}, {comp}; 0)")
            if len(pieces) > 4:
                raise NotImplementedError("more than 4 temperature ranges")
            for k, (lo, hi, coefs) in enumerate(pieces):
                table[ph, cp, k, 0], table[ph, cp, k, 1] = lo, hi
                table[ph, cp, k, 2:] = coefs
            npieces[ph, cp] = len(pieces)
    return table, npieces


def params_struct(db: Database, ud: dict, dx: float, noise_scale: float = 1.0,
                  variant: int = L.PPF_NCGPU_VARIANT_NCGPU):
    """PpfNcgpuParams from the derived parameters `ud` (ncgpu_parameters)
    and the database's Gibbs-energy tables. variant PPF_NCGPU_VARIANT_NEW
    (NCGPU_new) takes eqbar, noise_phi and noise_q from `ud`; noise_scale is
    the concentration noise's amplitude."""
    table, npieces = gibbs_table(db)
    p = L.PpfNcgpuParams()
    p.variant = int(variant)
    if variant == L.PPF_NCGPU_VARIANT_NEW:
        p.eqbar2 = float(ud["eqbar"]) * float(ud["eqbar"])
        p.noise_phi = float(ud["noise_phi"])
        p.noise_q = float(ud["noise_q"])
    for name in ("dt", "v_m", "D_L", "D_S", "M_qmax", "H", "y_e", "beta"):
        setattr(p, name, float(ud[name]))
    p.dx = float(dx)
    p.ebar2 = float(ud["ebar"]) * float(ud["ebar"])
    p.noise_scale = float(noise_scale)
    p.ncomp = len(db.elements)
    for j in range(p.ncomp):
        p.W[j] = float(ud["W"][j])
        p.M[j] = float(ud["M"][j])
    for ph in range(2):
        for cp in range(L.PPF_NCGPU_MAX_COMP):
            p.npieces[ph][cp] = int(npieces[ph, cp])
            for k in range(4):
                for e in range(10):
                    p.gibbs[ph][cp][k][e] = float(table[ph, cp, k, e])
    terms = excess_terms(db)
    p.nexcess = len(terms)
    for j, (phase, a, b, order, pieces) in enumerate(terms):
        x = p.excess[j]
        x.phase, x.a, x.b, x.order, x.npieces = phase, a, b, order, len(pieces)
        for k, (lo, hi, coefs) in enumerate(pieces):
            x.piece[k][0], x.piece[k][1] = lo, hi
            for e, v in enumerate(coefs):
                x.piece[k][2 + e] = float(v)
    return p


def excess_terms(db: Database) -> list:
    """The database's binary Redlich-Kister terms as (phase index (0 the
    solid, 1 the liquid), component index a, b, order, pieces)."""
    out = []
    for phase, a, b, order, pieces in db.excess:
        if phase not in db.phases:
            raise ValueError(f"L({phase},{a},{b};{order}): phase not listed")
        if len(pieces) > 4:
            raise NotImplementedError("more than 4 temperature ranges")
        out.append((db.phases.index(phase), db.elements.index(a), db.elements.index(b), order,
                    pieces))
    if len(out) > L.PPF_NCGPU_MAX_EXCESS:
        raise NotImplementedError(f"NCGPU: at most {L.PPF_NCGPU_MAX_EXCESS} interaction terms "
                                  f"(the TDB has {len(out)})")
    return out


def make_seed(phi, q1, q4, x, y, angle, seed_radius):
    """phi = 1 within seed_radius of (x, y), the quaternion at `angle` within
    seed_radius + 5 (NCGPU.make_seed, :305-320; half angles, periodic wrap)."""
    ny, nx = phi.shape
    qrad = seed_radius + 5
    yy, xx = np.mgrid[int(y - qrad):int(y + qrad), int(x - qrad):int(x + qrad)]
    r2 = (yy - y) ** 2 + (xx - x) ** 2
    inner = (yy >= int(y - seed_radius)) & (yy < int(y + seed_radius)) & \
        (xx >= int(x - seed_radius)) & (xx < int(x + seed_radius)) & (r2 < seed_radius ** 2)
    phi[yy[inner] % ny, xx[inner] % nx] = 1
    outer = r2 < qrad ** 2
    q1[yy[outer] % ny, xx[outer] % nx] = np.cos(0.5 * angle)
    q4[yy[outer] % ny, xx[outer] % nx] = np.sin(0.5 * angle)
    return phi, q1, q4


class _NcgpuMixin(GB300Engine):
    NFIELDS = 4
    VARIANT = L.PPF_NCGPU_VARIANT_NCGPU

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        self.user_data.setdefault("d_ratio", 4.0)
        self.user_data.setdefault("seed", 0)
        self.user_data.setdefault("noise_scale", 1.0)
        # float64 by default: the kernel's thresholds (|grad q| >= beta, the
        # phi clamp) flip for some cells in float32 within a few steps
        self.user_data.setdefault("precision", "fp64")
        self._ppf_defaults()
        self._ppf_db = None

    def init_tdb_params(self):
        if self._tdb_path is None:
            raise ValueError("NCGPU needs tdb_path (a thermodynamic database)")
        self._ppf_db = Database(self._tdb_path)
        if self.dx is None:
            raise ValueError("NCGPU needs dx")
        self.user_data.update(ncgpu_parameters(self._ppf_db, float(self.dx),
                                               float(self.user_data["d_ratio"])))
        self._tdb_components = list(self._ppf_db.elements)
        self._tdb_phases = list(self._ppf_db.phases)
        # phi, q1, q4 and all but the last component's fraction
        self.NFIELDS = 2 + len(self._tdb_components)
        self.dt = self.user_data["dt"]  # set_time_step_length (:367)

    def init_fields(self):
        dim = self.dimensions
        if len(dim) != 2:
            raise NotImplementedError("NCGPU runs 2-D grids (the reference's 1-D / 3-D paths "
                                      "launch its 2-D kernels)")
        ud = self.user_data
        comps = self._tdb_components
        phi = np.zeros(dim)
        melt = float(ud.get("melt_angle", 0.0)) if ud.get("sim_type") == "seed" else 0.0
        q1 = np.full(dim, np.cos(0.5 * melt))
        q4 = np.full(dim, np.sin(0.5 * melt))
        if ud.get("sim_type") == "seed":
            seed_angle = float(ud.get("seed_angle", np.pi / 4))
            phi, q1, q4 = make_seed(phi, q1, q4, dim[1] / 2, dim[0] / 2, seed_angle, 5)
        self.add_field(phi, "phi")
        self.add_field(q1, "q1")
        self.add_field(q4, "q4")
        self._add_concentrations()

    def _add_concentrations(self):
        """c_<component> for all but the last component: the
        initial_concentration_array, or 1 / N each when it is missing or has
        the wrong length (the reference's fallback, NCGPU.py:404-415)."""
        dim, comps = self.dimensions, self._tdb_components
        c0 = self.user_data.get("initial_concentration_array")
        if c0 is not None and len(c0) + 1 != len(comps):
            c0 = None
        for j in range(len(comps) - 1):
            val = float(c0[j]) if c0 is not None else 1.0 / len(comps)
            self.add_field(np.full(dim, val), "c_" + comps[j])

    def _ppf_prepare(self):
        t = self._temperature_type
        if self.temperature is None or t not in ("ISOTHERMAL", "LINEAR_GRADIENT"):
            raise ValueError("NCGPU needs an ISOTHERMAL or LINEAR_GRADIENT temperature field")
        if self._boundary_conditions_type is None:
            self._boundary_conditions_type = "PERIODIC"

    def _ppf_setup(self):
        super()._ppf_setup()
        g = self._ppf_grid
        self._nc_temp = g.empty()
        ncomp = len(self._tdb_components)
        self._nc_transfer = torch.zeros((2 * ncomp - 1,) + tuple(g.alloc_shape), dtype=g.dtype,
                                        device=g.device)
        # the pinned staging copy must outlive the asynchronous upload
        self._nc_temp_staging = self._ppf_grid.upload(self._nc_temp, self.temperature.get_cells(),
                                                      self._ppf_stream)
        ud = self.user_data
        noise = ud.get("noise_c", 1.0) if self.VARIANT else ud.get("noise_scale", 1.0)
        self._nc_params = params_struct(self._ppf_db, ud, self.dx, noise, self.VARIANT)
        self._nc_tables = None
        if not self._nc_dT():
            # a temperature fixed during the run: the pure-element energies of
            # every cell are evaluated once, after the upload, on the same
            # stream (with dT/dt every step evaluates them at its own T)
            nplanes = 2 * ncomp + int(self._nc_params.nexcess)
            self._nc_tables = torch.empty((nplanes,) + tuple(g.alloc_shape),
                                          dtype=torch.float64, device=g.device)
            L.call(f"ppf_ncgpu_tables_{_F[self._ppf_dtype]}", C.byref(self._nc_params),
                   C.byref(g.grid), ptr(self._nc_temp), ptr(self._nc_tables),
                   C.c_void_p(self._ppf_stream.cuda_stream))

    def _nc_dT(self) -> float:
        """Temperature rise per step, dTdt * dt (LINEAR_GRADIENT with dT/dt;
        else 0)."""
        if self._temperature_type == "LINEAR_GRADIENT" and self._dTdt:
            return float(self._dTdt) * float(self.dt)
        return 0.0

    def _ppf_send(self, s):
        super()._ppf_send(s)
        # the temperature field too: the host copy is the one that advances
        # with the step counter between runs
        if getattr(self, "_nc_temp", None) is not None:
            self._nc_temp_staging = self._ppf_grid.upload(self._nc_temp,
                                                          self.temperature.get_cells(), s)

    def _ppf_step(self, src, dst, depth, step, step_base, sp):
        fin = (C.c_void_p * len(src))(*[ptr(t) for t in src])
        fout = (C.c_void_p * len(dst))(*[ptr(t) for t in dst])
        L.call(f"ppf_ncgpu_step_{_F[self._ppf_dtype]}", C.byref(self._nc_params),
               C.byref(self._ppf_grid.grid), C.byref(self._ppf_bc), fin, fout,
               ptr(self._nc_temp), ptr(self._nc_tables), ptr(self._nc_transfer),
               C.c_uint64(int(self.user_data["seed"])),
               C.c_uint64(int(step)), ptr(step_base), sp)
        dT = self._nc_dT()
        if dT:
            # the step read T; then T rises (Simulation.simulate, simulation.py:262-266)
            L.call(f"ppf_ncgpu_temperature_advance_{_F[self._ppf_dtype]}",
                   C.byref(self._ppf_grid.grid), ptr(self._nc_temp), C.c_double(dT), sp)


class _NcgpuNewMixin(_NcgpuMixin):
    """NCGPU_new (Engines/NCGPU_new.py:340-553): the same fields and
    database, with a derivative dF/dc and a noise draw per component, phase
    noise sqrt(2 R T M_phi / v_m) scaled by user_data noise_phi, orientation
    noise sqrt(1e-10 R T / v_m) scaled by noise_q, concentration noise
    scaled by noise_c (all 1 by default), eqbar = 0.1 ebar and phi clamped
    to [1e-4, 0.9999]. The orientation starts at melt_angle for every
    sim_type; "seeds" places number_of_seeds seeds (default one per 10,000
    cells) at positions and angles from the engine's seeded generator
    (the reference draws them from numpy's global one)."""
    VARIANT = L.PPF_NCGPU_VARIANT_NEW

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        for key in ("noise_phi", "noise_c", "noise_q"):
            self.user_data.setdefault(key, 1.0)

    def init_tdb_params(self):
        super().init_tdb_params()
        self.user_data["eqbar"] = 0.1 * self.user_data["ebar"]  # NCGPU_new.py:385

    def init_fields(self):
        dim = self.dimensions
        if len(dim) != 2:
            raise NotImplementedError("NCGPU_new runs 2-D grids")
        ud = self.user_data
        melt = float(ud.get("melt_angle", 0.0))
        phi = np.zeros(dim)
        q1 = np.full(dim, np.cos(0.5 * melt))
        q4 = np.full(dim, np.sin(0.5 * melt))
        if ud.get("sim_type") == "seed":
            seed_angle = float(ud.get("seed_angle", np.pi / 4))
            phi, q1, q4 = make_seed(phi, q1, q4, dim[1] / 2, dim[0] / 2, seed_angle, 5)
        elif ud.get("sim_type") == "seeds":
            rng = np.random.default_rng(int(ud["seed"]))
            for _ in range(int(ud.get("number_of_seeds", int(np.prod(dim)) // 10000))):
                angle = (rng.random() - 0.5) * np.pi / 2 + melt
                x = int(rng.random() * dim[1])
                y = int(rng.random() * dim[0])
                phi, q1, q4 = make_seed(phi, q1, q4, x, y, angle, 5)
        self.add_field(phi, "phi")
        self.add_field(q1, "q1")
        self.add_field(q4, "q4")
        self._add_concentrations()


def make_ncgpu(base=Simulation):
    return type("NCGPUGB300", (_NcgpuMixin, base), {"__module__": __name__,
                                                   "__doc__": __doc__})


def make_ncgpu_new(base=Simulation):
    return type("NCGPU_newGB300", (_NcgpuNewMixin, base),
                {"__module__": __name__, "__doc__": _NcgpuNewMixin.__doc__})


NCGPUGB300 = make_ncgpu(Simulation)
NCGPU_newGB300 = make_ncgpu_new(Simulation)
