"""Runs pyphasefield's OWN numpy engine functions (TEST INFRASTRUCTURE ONLY).

The reference package imports matplotlib, meshio and tinydb at module level
(field.py:2, ppf_utils.py:1-6, simulation.py:3-9); none is needed by the
explicit engines, so this module installs inert stand-ins in sys.modules,
imports the reference from its checkout, and drives the module-level engine
functions with a duck-typed simulation object:

  * engine_ExplicitDiffusion (Engines/Diffusion.py:198-208) reads an
    undefined global ``self`` (:206): it is injected as the duck sim.
  * engine_CahnAllenExplicit / engine_CahnHilliardExplicit read an undefined
    global ``user_data`` (CahnAllen.py:131-133, CahnHilliard.py:138-140):
    injected.
  * engine_Warren1995 reads sim.W_A etc. as attributes (Warren1995.py:59-84):
    the duck sim carries them. Its np.random.random draw (:85) is replaced by
    a caller-supplied array through a numpy proxy in the module's globals.
  * The ghost fill between steps is oracle.restate.fill_ghosts (the
    reference's apply_boundary_conditions with every axis filled).
  * The implicit / Crank-Nicolson engines (Diffusion.py:210-633) run on an
    interior-only field (run_implicit).

Available only where the environment variable PPF_REFERENCE_ROOT names a
reference checkout (the directory holding the pyphasefield package); callers
skip otherwise. Nothing here is used at run time.
"""
from __future__ import annotations

import os
import sys
import types
from pathlib import Path

import numpy as np

from . import restate

def reference_root() -> Path | None:
    env = os.environ.get("PPF_REFERENCE_ROOT")
    if not env:
        return None
    root = Path(env)
    return root if (root / "pyphasefield" / "Engines" / "Warren1995.py").exists() else None


def available() -> bool:
    return reference_root() is not None


def _install_stubs() -> None:
    def mod(name):
        m = sys.modules.get(name)
        if m is None:
            m = types.ModuleType(name)
            sys.modules[name] = m
        return m

    mpl = mod("matplotlib")
    colors = mod("matplotlib.colors")
    cm = mod("matplotlib.cm")
    plt = mod("matplotlib.pyplot")

    class _Cmap:
        @staticmethod
        def from_list(*a, **k):
            return None

    colors.LinearSegmentedColormap = _Cmap
    colors.PowerNorm = lambda *a, **k: None
    mpl.colors, mpl.cm, mpl.pyplot = colors, cm, plt
    mod("meshio")
    mod("tinydb").where = lambda *a, **k: None


_MODS = None


def modules() -> dict:
    """Import the reference (with stand-ins) and return its engine modules."""
    global _MODS
    if _MODS is None:
        root = reference_root()
        if root is None:
            raise RuntimeError("reference checkout not found")
        _install_stubs()
        if str(root) not in sys.path:
            sys.path.insert(0, str(root))
        import io
        import contextlib
        with contextlib.redirect_stdout(io.StringIO()):  # numba-less engines print and skip
            import pyphasefield  # noqa: F401
            import pyphasefield.Engines  # noqa: F401
        _MODS = {k: sys.modules[f"pyphasefield.Engines.{k}"]
                 for k in ("Diffusion", "CahnAllen", "CahnHilliard", "Warren1995")}
        _MODS["field"] = sys.modules["pyphasefield.field"]
    return _MODS


class DuckSim:
    """The attributes the reference engine functions read from a Simulation."""

    def __init__(self, arrays, dx, dt, user_data=None, **attrs):
        Field = modules()["field"].Field
        self.dx = dx
        self.dt = dt
        self.user_data = dict(user_data or {})
        self.fields = []
        for a in arrays:
            f = Field(data=np.asarray(a, dtype=np.float64), simulation=self, name="f")
            self.fields.append(f)
        for k, v in attrs.items():
            setattr(self, k, v)

    def get_time_step_length(self):
        return self.dt

    def get_cell_spacing(self):
        return self.dx

    def get_dimensions(self):
        return list(self.fields[0].get_cells().shape)


class _NumpyWithNoise:
    """numpy stand-in whose random.random(shape) returns a fixed array."""

    def __init__(self, noise):
        self.random = types.SimpleNamespace(random=lambda shape: noise)

    def __getattr__(self, name):
        return getattr(np, name)


def run_single(model: str, c0, steps: int, boundary_conditions, dx: float,
               dt: float, values=None, **params) -> np.ndarray:
    """Drive the reference's one-field engine function for `steps` steps.
    For Cahn-Hilliard the reference has no dt: M*dt is passed as its M."""
    m = modules()
    sim = DuckSim([c0], dx, dt)
    bcs = restate.bc_list(boundary_conditions, np.ndim(c0))
    restate.fill_ghosts([f.data for f in sim.fields], bcs, dx, values)
    for _ in range(steps):
        if model == "diffusion":
            mod = m["Diffusion"]
            sim.user_data = {"D": params["D"]}
            mod.self = sim
            mod.engine_ExplicitDiffusion(sim)
        elif model == "allen_cahn":
            mod = m["CahnAllen"]
            mod.user_data = {k: params[k] for k in ("M", "W", "epsilon")}
            mod.engine_CahnAllenExplicit(sim)
        elif model == "cahn_hilliard":
            mod = m["CahnHilliard"]
            mod.user_data = {"M": params["M"] * dt, "W": params.get("W", 1.0),
                             "epsilon": params["epsilon"]}
            mod.engine_CahnHilliardExplicit(sim)
        else:
            raise ValueError(model)
        restate.fill_ghosts([f.data for f in sim.fields], bcs, dx, values)
    return sim.fields[0].get_cells().copy()


def run_cahn_hilliard_extended(c0, steps: int, boundary_conditions, dx: float,
                               dt: float, M: float, epsilon: float) -> np.ndarray:
    """Cahn-Hilliard through the reference's function with its mu-ghost
    defect kept away from the answer: the field is extended by 2*steps cells
    per side (periodic wrap or no-flux mirror, the exact continuation of
    those boundary rules), the reference advances the extended field, and the
    centre is cropped. The result is the reference's arithmetic on every
    cell that matters."""
    c0 = np.asarray(c0, dtype=np.float64)
    h = 2 * steps + 2
    bcs = restate.bc_list(boundary_conditions, c0.ndim)
    ext = c0
    for ax, b in enumerate(bcs):
        mode = "wrap" if b == restate.PERIODIC else "symmetric"
        widths = [(0, 0)] * c0.ndim
        widths[ax] = (h, h)
        ext = np.pad(ext, widths, mode=mode)
    out = run_single("cahn_hilliard", ext, steps, bcs, dx, dt, M=M, epsilon=epsilon)
    return out[(slice(h, -h),) * c0.ndim].copy()


def run_warren(phi0, c0, steps: int, boundary_conditions, dx: float, params: dict,
               noise=None, values=None):
    """Drive engine_Warren1995 for `steps` steps. noise: list of interior
    U[0,1) arrays, one per step (None: no noise term, alpha forced to 0)."""
    m = modules()
    mod = m["Warren1995"]
    p = restate.warren_derived(params, dx)
    attrs = {k: p[k] for k in ("W_A", "W_B", "L_A", "L_B", "T", "T_mA", "T_mB", "D_S",
                               "D_L", "v_m", "R", "y_e", "M_A", "M_B", "ebar")}
    attrs["alpha"] = p["alpha"] if noise is not None else 0.0
    sim = DuckSim([phi0, c0], dx, p["dt"], **attrs)
    bcs = restate.bc_list(boundary_conditions, 2)
    restate.fill_ghosts([f.data for f in sim.fields], bcs, dx, values)
    saved = mod.np
    try:
        for s in range(steps):
            u = restate.pad(noise[s]) if noise is not None else np.zeros(sim.fields[0].data.shape)
            mod.np = _NumpyWithNoise(u)
            mod.engine_Warren1995(sim)
            restate.fill_ghosts([f.data for f in sim.fields], bcs, dx, values)
    finally:
        mod.np = saved
    return sim.fields[0].get_cells().copy(), sim.fields[1].get_cells().copy()


class _InteriorSim:
    """A simulation whose one Field holds the interior cells only: the
    reference's implicit engines size their matrices by get_dimensions()
    (the interior) and solve against Field.data, so they run as written on
    it; Field.laplacian then wraps periodically, as the matrices do."""

    def __init__(self, c, dx, dt, D=None):
        Field = modules()["field"].Field
        f = Field(data=np.asarray(c, dtype=np.float64), simulation=self, name="c")
        f.data = np.array(c, dtype=np.float64)
        self.fields = [f]
        self.dx, self.dt = dx, dt
        self.user_data = {"D": D}
        self._dims = list(np.shape(c))

    def get_cell_spacing(self):
        return self.dx

    def get_dimensions(self):
        return list(self._dims)


def _gmres_legacy(A, b, atol=None, **kw):
    """scipy.sparse.linalg.gmres with the meaning atol='legacy' had (a
    residual bound of 1e-5 relative to |b|): scipy 1.14 and later reject
    'legacy', which makes every *_GMRES engine raise as written."""
    from scipy.sparse.linalg import gmres
    return gmres(A, b, rtol=1e-5, atol=0.0)


def run_implicit(function: str, c0, steps: int, D: float, dt: float, dx: float,
                 module: str = "Diffusion", user_data=None) -> np.ndarray:
    """Drive one of the reference's implicit / Crank-Nicolson / IMEX engine
    functions (Diffusion.py:210-633, CahnAllen.py:137-267,
    CahnHilliard.py:148-341) for `steps` steps on the interior array. The
    module globals they read (``self`` in Diffusion.py, ``user_data`` in the
    other two) are injected; the *_GMRES functions get _gmres_legacy."""
    mod = modules()[module]
    sim = _InteriorSim(c0, dx, dt, D)
    saved = mod.gmres
    mod.self = sim
    if user_data is not None:
        mod.user_data = dict(user_data)
    mod.gmres = _gmres_legacy
    try:
        fn = getattr(mod, function)
        for _ in range(steps):
            fn(sim)
    finally:
        mod.gmres = saved
    return np.array(sim.fields[0].data, dtype=np.float64).reshape(np.shape(c0))


# ---------------------------------------------------------------------------
# NCGPU (Engines/NCGPU.py): its kernels are numba CUDA kernels written as
# grid-stride loops, so with a stand-in numba module (cuda.jit = the plain
# function, cuda.grid = 0, cuda.gridsize = 1) each runs as one Python loop
# over the whole grid: the reference's own arithmetic, serially.

def _install_numba_standin(normal_source):
    import types as _t

    def jit(*a, **k):
        if a and callable(a[0]):
            return a[0]
        return lambda f: f

    numba = _t.ModuleType("numba")
    cuda = _t.ModuleType("numba.cuda")
    rnd = _t.ModuleType("numba.cuda.random")
    numba.jit = jit
    cuda.jit = jit
    cuda.grid = lambda n: (0, 0) if n == 2 else 0
    cuda.gridsize = lambda n: (1, 1) if n == 2 else 1
    cuda.synchronize = lambda: None
    rnd.create_xoroshiro128p_states = lambda n, seed=0: None
    rnd.xoroshiro128p_uniform_float32 = lambda states, tid: 0.5
    rnd.xoroshiro128p_normal_float32 = lambda states, tid: normal_source()
    cuda.random = rnd
    numba.cuda = cuda
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = cuda
    sys.modules["numba.cuda.random"] = rnd


_NC = {"queue": None}


def ncgpu_module(name: str = "NCGPU"):
    """Import Engines/NCGPU.py (or NCGPU_new.py) with the numba stand-in
    (test use only)."""
    full = "pyphasefield.Engines." + name
    mod = sys.modules.get(full)
    if mod is not None and getattr(mod, "_ppf_standin", False):
        return mod

    def normal():
        q = _NC["queue"]
        return next(q) if q is not None else 0.0

    saved = {k: sys.modules.get(k) for k in ("numba", "numba.cuda", "numba.cuda.random")}
    modules()
    _install_numba_standin(normal)
    try:
        import importlib
        sys.modules.pop(full, None)
        mod = importlib.import_module(full)
        mod._ppf_standin = True
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod


def run_ncgpu(phi, q1, q4, c, T, steps: int, p: dict, tdb, noise_fields, bc="PERIODIC",
              dT_step=0.0):
    """Drive NComponent_helper_kernel and NComponent_kernel for `steps`
    steps; c is one concentration field (binary) or a list of N - 1 of them.
    noise_fields[s] is the interior N(0,1) field of step s; ghost cells take
    the noise of the cell the boundary rule maps them to. Ghost cells of
    every field and of T follow `bc` (PERIODIC or zero-gradient NEUMANN), as
    ppf_gpu_utils.apply_boundary_conditions fills them between steps.
    dT_step (dTdt * dt of a LINEAR_GRADIENT temperature): after every step
    each cell of the padded temperature array rises by it, as
    update_thermal_gradient_2D_kernel (ppf_gpu_utils.py:326-334) does."""
    mod = ncgpu_module()
    mode = "wrap" if bc == "PERIODIC" else "symmetric"
    pad = lambda a: np.pad(np.asarray(a, dtype=np.float64), 1, mode=mode)  # noqa: E731
    cs = [np.array(x, dtype=np.float64) for x in (c if isinstance(c, (list, tuple)) else [c])]
    f = [np.array(a, dtype=np.float64) for a in (phi, q1, q4)] + cs
    ncomp = len(cs) + 1
    ny, nx = f[0].shape
    Tp = pad(T)
    params = np.array([p["dx"], p["d"], p["v_m"], p["M_qmax"], p["H"], p["y_e"], p["beta"],
                       p["D_L"], p["D_S"], p["dt"]])
    c_params = np.array([p["L"], p["T_M"], p["S"], p["B"], p["W"], p["M"]])
    phases = tdb.phases
    mod.ufunc_g_l = lambda arr: tdb.gibbs(phases[1], list(arr[:ncomp]), arr[ncomp])
    mod.ufunc_g_s = lambda arr: tdb.gibbs(phases[0], list(arr[:ncomp]), arr[ncomp])
    for s in range(steps):
        fields = np.stack([pad(a) for a in f])
        out = np.zeros_like(fields)
        transfer = np.zeros((2 * ncomp,) + fields.shape[1:])
        ufunc_array = np.zeros(fields.shape[1:] + (ncomp + 1,))
        nz = pad(noise_fields[s])
        _NC["queue"] = iter(nz.ravel().tolist())
        mod.NComponent_helper_kernel(fields, Tp, transfer, None, ufunc_array, params, c_params)
        _NC["queue"] = iter([0.0] * (ny * nx))
        mod.NComponent_kernel(fields, Tp, transfer, out, None, params, c_params)
        f = [out[k, 1:-1, 1:-1].copy() for k in range(len(f))]
        if dT_step:
            Tp += dT_step
    _NC["queue"] = None
    return f


def run_ncgpu_new(phi, q1, q4, c, T, steps: int, p: dict, tdb, noise, bc="PERIODIC"):
    """Drive NCGPU_new's helper and main kernels (Engines/NCGPU_new.py:38-314)
    for `steps` steps. noise[s] is oracle.ncgpu_ref.noise_new's dict for step
    s: the helper draws one normal per concentration field and cell (ghost
    cells take the draw of the cell the boundary rule maps them to), the
    main kernel three per interior cell (phase, q1, q4) in its own loop order
    (columns outer, rows inner)."""
    mod = ncgpu_module("NCGPU_new")
    mode = "wrap" if bc == "PERIODIC" else "symmetric"
    pad = lambda a: np.pad(np.asarray(a, dtype=np.float64), 1, mode=mode)  # noqa: E731
    cs = [np.array(x, dtype=np.float64) for x in (c if isinstance(c, (list, tuple)) else [c])]
    f = [np.array(a, dtype=np.float64) for a in (phi, q1, q4)] + cs
    ncomp = len(cs) + 1
    Tp = pad(T)
    params = np.array([p["dx"], p["d"], p["v_m"], p["M_qmax"], p["H"], p["y_e"], p["beta"],
                       p["D_L"], p["D_S"], p["dt"], p["ebar"], p["eqbar"], p["noise_phi"],
                       p["noise_c"], p["noise_q"]])
    c_params = np.array([p["L"], p["T_M"], p["S"], p["B"], p["W"], p["M"]])
    phases = tdb.phases
    mod.ufunc_g_l = lambda arr: tdb.gibbs(phases[1], list(arr[:ncomp]), arr[ncomp])
    mod.ufunc_g_s = lambda arr: tdb.gibbs(phases[0], list(arr[:ncomp]), arr[ncomp])
    for s in range(steps):
        fields = np.stack([pad(a) for a in f])
        out = np.zeros_like(fields)
        transfer = np.zeros((2 * ncomp,) + fields.shape[1:])
        ufunc_array = np.zeros(fields.shape[1:] + (ncomp + 1,))
        nzc = np.stack([pad(a) for a in noise[s]["c"]], axis=-1)  # (rows, cols, component)
        _NC["queue"] = iter(nzc.ravel().tolist())
        mod.NComponent_helper_kernel(fields, Tp, transfer, None, ufunc_array, params, c_params)
        nzm = np.stack([noise[s][k] for k in ("phi", "q1", "q4")], axis=-1)  # interior
        _NC["queue"] = iter(np.transpose(nzm, (1, 0, 2)).ravel().tolist())
        mod.NComponent_kernel(fields, Tp, transfer, out, None, params, c_params)
        f = [out[k, 1:-1, 1:-1].copy() for k in range(len(f))]
    _NC["queue"] = None
    return f
