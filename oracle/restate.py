"""FP64 numpy restatement of pyphasefield's explicit hot path.

TEST INFRASTRUCTURE ONLY. This module is the oracle: tests, the smoke check
and the CPU-baseline leg of the benchmark use it to check the CUDA library.
Nothing in the shipped package imports it.

Every function follows the reference's own numpy code on ghost-padded arrays
(one ghost layer per side, as pyphasefield.field.Field stores them), with the
ghost fill of Simulation.apply_boundary_conditions applied on every axis. The
deviations from the literal reference are the reference's defects, corrected
(each is named where it happens):
  * simulation.py:561-566 builds the slice for axis k >= 1 as (None, ..., k),
    which indexes a new axis and never fills the ghosts of axes >= 1; here the
    slice selects index k along axis k.
  * Engines/CahnHilliard.py:134-146 omits dt and takes the Laplacian of mu by
    np.roll over the padded array, so ghost mu values are built from wrapped
    ghost c values; here mu ghosts are refilled with the field's boundary rule
    (periodic wrap / no-flux mirror) before the second Laplacian, and dt*M
    multiplies it.
Parity of this restatement with the reference's own functions is checked by
tests/test_oracle.py through oracle/refshim.py (in a checkout that has the
reference) and pinned by the committed vectors in tests/golden/.
"""
from __future__ import annotations

import numpy as np

PERIODIC, NEUMANN, DIRCHLET = "PERIODIC", "NEUMANN", "DIRCHLET"


def bc_list(boundary_conditions, ndim: int) -> list[str]:
    """Per-axis list of boundary types, as Simulation.apply_boundary_conditions
    accepts them (a single string or one string per axis)."""
    if isinstance(boundary_conditions, str):
        return [boundary_conditions] * ndim
    bc = list(boundary_conditions)
    if len(bc) != ndim:
        raise ValueError(f"need {ndim} boundary types, got {bc}")
    return bc


def pad(interior: np.ndarray) -> np.ndarray:
    """Zero ghost layer around the interior, like Field.__init__ (field.py:6-20)."""
    out = np.zeros([n + 2 for n in interior.shape])
    out[(slice(1, -1),) * interior.ndim] += interior
    return out


def interior(padded: np.ndarray) -> np.ndarray:
    """Field.get_cells (field.py:69-70)."""
    return padded[(slice(1, -1),) * padded.ndim]


def fill_ghosts(fields, boundary_conditions, dx: float, values=None) -> None:
    """Ghost fill of Simulation.apply_boundary_conditions (simulation.py:560-618),
    axis by axis in the reference's order, with every axis filled.

    values[j][axis][side] is field j's Neumann gradient or Dirichlet value on
    that face (the reference keeps it in _boundary_conditions_array; default 0).
    """
    nd = fields[0].ndim
    bcs = bc_list(boundary_conditions, nd)

    def at(axis, k):
        return (slice(None),) * axis + (k,)

    for i in range(nd):
        for j, f in enumerate(fields):
            lo = values[j][i][0] if values is not None else 0.0
            hi = values[j][i][1] if values is not None else 0.0
            if bcs[i] == PERIODIC:
                f[at(i, 0)] = f[at(i, -2)]
                f[at(i, -1)] = f[at(i, 1)]
            elif bcs[i] == NEUMANN:
                f[at(i, 0)] = f[at(i, 1)] - dx * lo
                f[at(i, -1)] = f[at(i, -2)] + dx * hi
            elif bcs[i] == DIRCHLET:
                f[at(i, 0)] = lo
                f[at(i, -1)] = hi
            else:
                raise ValueError(f"unknown boundary condition {bcs[i]!r}")


def laplacian(data: np.ndarray, dx: float) -> np.ndarray:
    """Field.laplacian (field.py:60-67): rolls over the padded array."""
    inv_dx2 = (1.0 / dx) ** 2
    out = (np.roll(data, -1, 0) + np.roll(data, 1, 0) - 2 * data) * inv_dx2
    for i in range(1, data.ndim):
        out += (np.roll(data, -1, i) + np.roll(data, 1, i) - 2 * data) * inv_dx2
    return out


# ----------------------------------------------------------------- engines
def diffusion_step(c: np.ndarray, dx: float, dt: float, D: float) -> None:
    """engine_ExplicitDiffusion (Engines/Diffusion.py:198-208), in place."""
    dc = dt * (D * laplacian(c, dx))
    c += dc


def allen_cahn_step(phi: np.ndarray, dx: float, dt: float, M: float,
                    epsilon: float, W: float) -> None:
    """engine_CahnAllenExplicit (Engines/CahnAllen.py:128-135), in place."""
    dphi = dt * M * (epsilon ** 2 * laplacian(phi, dx)
                     - 16.0 * W * (4.0 * phi ** 3 - 6.0 * phi ** 2 + 2.0 * phi))
    phi += dphi


def cahn_hilliard_step(c: np.ndarray, dx: float, dt: float, M: float,
                       epsilon: float, boundary_conditions) -> None:
    """engine_CahnHilliardExplicit (Engines/CahnHilliard.py:134-146), in place,
    with dt applied and mu's ghosts refilled by the boundary rule (no-flux for
    NEUMANN axes) before its Laplacian."""
    mu = -epsilon ** 2 * laplacian(c, dx) + (4 * c ** 3 - 6 * c ** 2 + 2 * c)
    bcs = bc_list(boundary_conditions, c.ndim)
    if DIRCHLET in bcs:
        raise ValueError("Cahn-Hilliard oracle supports PERIODIC and NEUMANN axes")
    fill_ghosts([mu], bcs, dx)
    dmu = 0
    for i in range(c.ndim):
        dmu = dmu + (np.roll(mu, 1, i) + np.roll(mu, -1, i) - 2 * mu)
    dmu = dmu / dx ** 2
    c += dt * M * dmu


WARREN_DEFAULTS = dict(
    T_mA=1728.0, T_mB=1358.0, L_A=2350000000.0, L_B=1728000000.0, s_A=0.37,
    s_B=0.29, D_L=1e-9, D_S=1e-13, B_A=0.0033, B_B=0.0039, v_m=0.00000742,
    R=8.314, y_e=0.04, T=1574.0, alpha=0.3)
"""Warren1995 user_data defaults (Engines/Warren1995.py:138-167)."""


def warren_derived(ud: dict, dx: float) -> dict:
    """Warren1995.just_before_simulating (Engines/Warren1995.py:193-203):
    dt and the derived interface/mobility constants."""
    out = dict(ud)
    out["dt"] = dx ** 2 / 5.0 / ud["D_L"]
    d = dx / 0.94
    out["d"] = d
    out["ebar"] = np.sqrt(6 * np.sqrt(2) * ud["s_A"] * d / ud["T_mA"])
    out["W_A"] = 3 * ud["s_A"] / (np.sqrt(2) * ud["T_mA"] * d)
    out["W_B"] = 3 * ud["s_B"] / (np.sqrt(2) * ud["T_mB"] * d)
    out["M_A"] = (ud["T_mA"] ** 2) * ud["B_A"] / (6 * np.sqrt(2) * ud["L_A"] * d)
    out["M_B"] = (ud["T_mB"] ** 2) * ud["B_B"] / (6 * np.sqrt(2) * ud["L_B"] * d)
    return out


def _gradx(f, dx):
    return (np.roll(f, 1, 0) - np.roll(f, -1, 0)) / (2 * dx)


def _grady(f, dx):
    return (np.roll(f, 1, 1) - np.roll(f, -1, 1)) / (2 * dx)


def _gradxx(f, dx):
    return (np.roll(f, 1, 0) + np.roll(f, -1, 0) - 2 * f) / (dx * dx)


def _gradyy(f, dx):
    return (np.roll(f, 1, 1) + np.roll(f, -1, 1) - 2 * f) / (dx * dx)


def warren1995_step(phi: np.ndarray, c: np.ndarray, p: dict, dx: float,
                    dt: float, noise_u: np.ndarray | None = None) -> None:
    """engine_Warren1995 (Engines/Warren1995.py:50-92), in place on padded
    phi and c. `p` holds the user_data constants plus ebar, W_A, W_B, M_A,
    M_B. noise_u (padded shape, values in [0, 1)) replaces the reference's
    np.random.random(phi.shape) draw (:85); None means zero noise."""
    g = phi * phi * (1 - phi) * (1 - phi)                      # _g (:20-21)
    pp = phi * phi * phi * (10 - 15 * phi + 6 * phi * phi)     # _p (:17-18)
    gprime = 4 * phi * phi * phi - 6 * phi * phi + 2 * phi     # _gprime (:23-24)
    H_A = p["W_A"] * gprime + 30 * p["L_A"] * (1 / p["T"] - 1 / p["T_mA"]) * g
    H_B = p["W_B"] * gprime + 30 * p["L_B"] * (1 / p["T"] - 1 / p["T_mB"]) * g
    phixx = _gradxx(phi, dx)
    phiyy = _gradyy(phi, dx)
    lphi = phixx + phiyy
    phix = _gradx(phi, dx)
    phiy = _grady(phi, dx)
    phixy = _grady(phix, dx)

    D_C = p["D_S"] + pp * (p["D_L"] - p["D_S"])
    temp = D_C * p["v_m"] * c * (1 - c) * (H_B - H_A) / p["R"]
    deltac = (D_C * (_gradxx(c, dx) + _gradyy(c, dx))
              + (_gradx(D_C, dx) * _gradx(c, dx) + _grady(D_C, dx) * _grady(c, dx))
              + temp * lphi
              + (_gradx(temp, dx) * phix + _grady(temp, dx) * phiy))

    theta = np.arctan2(phiy, phix)
    eta = 1 + p["y_e"] * np.cos(4 * theta)
    etap = -4 * p["y_e"] * np.sin(4 * theta)
    etapp = -16 * (eta - 1)
    c2 = np.cos(2 * theta)
    s2 = np.sin(2 * theta)
    M_phi = (1 - c) * p["M_A"] + c * p["M_B"]
    ebar2 = p["ebar"] ** 2
    deltaphi = M_phi * ((ebar2 * eta * eta * lphi - (1 - c) * H_A - c * H_B)
                        + ebar2 * eta * etap * (s2 * (phiyy - phixx) + 2 * c2 * phixy)
                        + 0.5 * ebar2 * (etap * etap + eta * etapp)
                        * (-2 * s2 * phixy + lphi + c2 * (phiyy - phixx)))
    if noise_u is not None and p["alpha"] != 0:
        rand = 2 * noise_u - 1
        deltaphi += M_phi * p["alpha"] * rand * (16 * g) * ((1 - c) * H_A + c * H_B)
    phi += deltaphi * dt
    c += deltac * dt


# ----------------------------------------------------------------- drivers
def run_single(model: str, c0: np.ndarray, steps: int, boundary_conditions,
               dx: float, dt: float, values=None, **params) -> np.ndarray:
    """Simulation.simulate (simulation.py:245-271) for a one-field model:
    ghost fill, then per step: engine step, ghost fill. Returns the interior."""
    c = pad(np.asarray(c0, dtype=np.float64))
    fill_ghosts([c], boundary_conditions, dx, values)
    for _ in range(steps):
        if model == "diffusion":
            diffusion_step(c, dx, dt, params["D"])
        elif model == "allen_cahn":
            allen_cahn_step(c, dx, dt, params["M"], params["epsilon"], params["W"])
        elif model == "cahn_hilliard":
            cahn_hilliard_step(c, dx, dt, params["M"], params["epsilon"], boundary_conditions)
        else:
            raise ValueError(model)
        fill_ghosts([c], boundary_conditions, dx, values)
    return interior(c).copy()


def run_warren(phi0: np.ndarray, c0: np.ndarray, steps: int, boundary_conditions,
               dx: float, params: dict, seed: int = 0, step0: int = 0,
               values=None) -> tuple[np.ndarray, np.ndarray]:
    """Warren1995 run: `params` are user_data constants; dt and the derived
    constants come from warren_derived. Noise uses the project's Philox
    stream (oracle.philox.noise_uniform) keyed by (seed, step) when
    params['alpha'] != 0."""
    from .philox import noise_uniform

    p = warren_derived(params, dx)
    phi = pad(np.asarray(phi0, dtype=np.float64))
    c = pad(np.asarray(c0, dtype=np.float64))
    fill_ghosts([phi, c], boundary_conditions, dx, values)
    for s in range(steps):
        noise = None
        if p["alpha"] != 0:
            noise = pad(noise_uniform(seed, step0 + s, phi0.shape))
        warren1995_step(phi, c, p, dx, p["dt"], noise)
        fill_ghosts([phi, c], boundary_conditions, dx, values)
    return interior(phi).copy(), interior(c).copy()
