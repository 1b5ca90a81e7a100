"""CPU restatement of pyphasefield's NCGPU engine (test infrastructure: only
tests/ and bench.py's CPU legs use it).

Reference: Engines/NCGPU.py
  NComponent_helper_kernel :248-303  thermodynamics, mobility and dF/dc per cell
  NComponent_kernel        :37-242   phi, quaternion (q1, q4) and c updates
  NCGPU.init_tdb_params    :336-373  parameters from the TDB file
  NCGPU.init_fields        :375-474  the single-seed initial condition
  simulation_loop          :499-532  helper, then kernel, then swap

The Gibbs energies are what pyphasefield builds with pycalphad
(simulation.py:179-243 / ppf_utils.TDBContainer): for each phase the
Redlich-Kister sum of the TDB's G and binary L parameters plus pycalphad's
ideal mixing energy R T sum x ln x, R = 8.3145 (pycalphad's
gas constant), evaluated at (x_1 .. x_N, T) with components and phases in
sorted order. pycalphad is not installed here; this module parses the TDB
FUNCTION / PARAMETER records it needs itself (`Tdb`). The reference kernel
itself runs unmodified under oracle/refshim.run_ncgpu (a stand-in numba
module); tests/golden/make_golden.py pins `step` below to it.

Restatement notes:
  * dG/dc: the reference takes a forward difference with step 1e-7 in
    float64 (:283-286); here (and on the GPU) the same difference is taken.
  * excess energies: binary Redlich-Kister L parameters are added in the
    CALPHAD convention (constituents in the order the record writes them);
    pycalphad, absent here, is the reference's evaluator of these terms.
  * noise: the reference draws N(0,1) per cell from numba's xoroshiro128p
    streams indexed by the x thread index only (:290); here a normal per
    (cell, step) from Philox4x32-10 by Box-Muller (`noise_normal`), the same
    numbers the GPU draws. Ghost cells take the noise of the interior cell
    the boundary rule maps them to (the reference draws independent numbers
    for ghost cells).
  * the reference computes noise_phi but never adds it (:183); it is not
    drawn here.
"""
from __future__ import annotations

import math
import re
from pathlib import Path

import numpy as np

from .philox import philox4x32_10

R_PYCALPHAD = 8.3145
R_KERNEL = 8.314  # the constant the kernels write out (:185, :290, :299)


class Tdb:
    """The FUNCTION and PARAMETER records of a TDB file (piecewise
    polynomials in T, with LN(T))."""

    def __init__(self, path):
        text = Path(path).read_text()
        # records end with '!'; comments start with '$'
        lines = [ln.split("$", 1)[0] for ln in text.splitlines()]
        records = " ".join(lines).split("!")
        self.functions: dict[str, list] = {}
        self.params: dict[tuple, str] = {}
        # binary Redlich-Kister terms: (phase, A, B, order k, pieces)
        self.excess: list[tuple] = []
        self.elements: list[str] = []
        self.phases: list[str] = []
        for rec in records:
            toks = rec.split()
            if not toks:
                continue
            kw = toks[0].upper()
            if kw == "ELEMENT":
                el = toks[1].upper()
                if el not in ("/-", "VA"):
                    self.elements.append(el)
            elif kw == "PHASE":
                self.phases.append(toks[1].upper().split(":")[0])  # LIQUID:L -> LIQUID
            elif kw == "FUNCTION":
                self.functions[toks[1].upper()] = self._pieces(" ".join(toks[2:]))
            elif kw == "PARAMETER":
                m = re.match(r"\s*PARAMETER\s+G\s*\(\s*([^,]+)\s*,\s*([^;]+);\s*0\s*\)\s*(.*)",
                             rec, re.IGNORECASE)
                if m:
                    phase = m.group(1).strip().upper()
                    comp = m.group(2).strip().upper()
                    body = self._pieces(m.group(3))
                    self.params[(phase, comp)] = body
                    continue
                m = re.match(r"\s*PARAMETER\s+L\s*\(\s*([^,]+?)\s*,\s*([^,;:]+?)\s*,"
                             r"\s*([^,;:]+?)\s*;\s*(\d+)\s*\)\s*(.*)", rec, re.IGNORECASE)
                if m:
                    self.excess.append((m.group(1).upper(), m.group(2).upper(),
                                        m.group(3).upper(), int(m.group(4)),
                                        self._pieces(m.group(5))))
        self.elements.sort()
        self.phases.sort()

    @staticmethod
    def _pieces(body: str):
        """'T0 expr1; T1 Y expr2; T2 N' -> [(T0, T1, expr1), (T1, T2, expr2)]."""
        parts = [p.strip() for p in body.split(";")]
        first = parts[0].split(None, 1)
        lo = float(first[0])
        expr = first[1]
        out = []
        for p in parts[1:]:
            toks = p.split(None, 2)
            hi = float(toks[0])
            out.append((lo, hi, expr.strip()))
            if len(toks) >= 2 and toks[1].upper() == "Y" and len(toks) == 3:
                lo, expr = hi, toks[2]
            else:
                break
        return out

    def value(self, name: str, T: float, _depth=0) -> float:
        """Value of FUNCTION `name` at temperature T (0 outside its ranges,
        as pycalphad's Piecewise gives)."""
        for lo, hi, expr in self.functions[name.upper()]:
            if lo <= T < hi:
                return self._eval(expr, T, _depth)
        return 0.0

    def _eval(self, expr: str, T: float, depth: int) -> float:
        if depth > 8:
            raise ValueError("TDB function nesting too deep")
        e = re.sub(r"LN\(", "log(", expr.replace("#", ""), flags=re.IGNORECASE)
        e = e.replace("e+0", "e+").replace("e-0", "e-")
        names = {"T": T, "log": math.log}
        for sym in set(re.findall(r"[A-Za-z_][A-Za-z_0-9]*", e)):
            if sym in names:
                continue
            if sym.upper() in self.functions:
                names[sym] = self.value(sym, T, depth + 1)
        return float(eval(e, {"__builtins__": {}}, names))

    def g_pure(self, phase: str, comp: str, T: float) -> float:
        for lo, hi, expr in self.params[(phase.upper(), comp.upper())]:
            if lo <= T < hi:
                return self._eval(expr, T, 0)
        return 0.0

    def excess_value(self, pieces, T: float) -> float:
        for lo, hi, expr in pieces:
            if lo <= T < hi:
                return self._eval(expr, T, 0)
        return 0.0

    def gibbs(self, phase: str, x, T: float) -> float:
        """Molar Gibbs energy of `phase` at site fractions x (components in
        sorted order): sum x_i G_i + R T sum x_i ln x_i + the binary
        Redlich-Kister terms x_A x_B L_k(T) (x_A - x_B)^k, A and B in the
        order the PARAMETER record writes them (the CALPHAD convention for
        odd k)."""
        g = 0.0
        for comp, xi in zip(self.elements, x):
            g += xi * self.g_pure(phase, comp, T)
        mix = sum(xi * math.log(xi) for xi in x if xi > 0)
        g = g + R_PYCALPHAD * T * mix
        for ph, a, b, k, pieces in self.excess:
            if ph != phase.upper():
                continue
            xa, xb = x[self.elements.index(a)], x[self.elements.index(b)]
            g += xa * xb * self.excess_value(pieces, T) * (xa - xb) ** k
        return g

    def scalar(self, name: str) -> float:
        """A constant FUNCTION (CU_L, V_M, ...) evaluated as npvalue does
        (at T = 1000, NCGPU.py:322-327)."""
        return self.value(name, 1000.0)


def tdb_params(tdb: Tdb, dx: float, d_ratio: float = 4.0, variant: str = "NCGPU") -> dict:
    """NCGPU.init_tdb_params (:336-373); variant "NCGPU_new" as
    NCGPU_new.init_tdb_params (NCGPU_new.py:350-386): eqbar = 0.1 ebar and
    the noise amplitudes noise_phi / noise_c / noise_q (1 by default)."""
    comps = tdb.elements
    d = dx * d_ratio
    p = {"d": d, "R": 8.314}
    for key in ("L", "TM", "S", "B"):
        p[key] = [tdb.scalar(f"{c}_{key}") for c in comps]
    p["T_M"] = p.pop("TM")
    p["W"] = [3 * s / (np.sqrt(2) * tm * d) for s, tm in zip(p["S"], p["T_M"])]
    p["M"] = [(tm ** 2) * b / (6 * np.sqrt(2) * lat * d) / 1574.0
              for tm, b, lat in zip(p["T_M"], p["B"], p["L"])]
    p["D_S"] = tdb.scalar("D_S")
    p["D_L"] = tdb.scalar("D_L")
    p["v_m"] = tdb.scalar("V_M")
    p["M_qmax"] = tdb.scalar("M_Q")
    p["H"] = tdb.scalar("H")
    p["y_e"] = tdb.scalar("Y_E")
    p["ebar"] = np.sqrt(6 * np.sqrt(2) * p["S"][1] * d / p["T_M"][1])
    p["eqbar"] = (0.1 if variant == "NCGPU_new" else 0.5) * p["ebar"]
    if variant == "NCGPU_new":
        p.update(noise_phi=1.0, noise_c=1.0, noise_q=1.0)
    p["dt"] = dx ** 2 / 5.0 / p["D_L"] / 8
    p["beta"] = 1.5
    p["dx"] = dx
    return p


def seed_fields(shape, melt_angle=0.0, seed_angle=np.pi / 4, radius=5, c0=None, ncomp=2):
    """NCGPU.init_fields with sim_type "seed" (:375-415) and make_seed
    (:305-320): phi = 1 in a disk of `radius` at the centre, quaternion
    angle seed_angle within radius + 5, melt_angle elsewhere; c = c0 (or
    1 / N for every listed component)."""
    phi = np.zeros(shape)
    q1 = np.full(shape, np.cos(0.5 * melt_angle))
    q4 = np.full(shape, np.sin(0.5 * melt_angle))
    y, x = shape[0] / 2, shape[1] / 2
    ny, nx = shape
    for i in range(int(y - radius), int(y + radius)):
        for j in range(int(x - radius), int(x + radius)):
            if (i - y) ** 2 + (j - x) ** 2 < radius ** 2:
                phi[i % ny, j % nx] = 1
    qr = radius + 5
    for i in range(int(y - qr), int(y + qr)):
        for j in range(int(x - qr), int(x + qr)):
            if (i - y) ** 2 + (j - x) ** 2 < qr ** 2:
                q1[i % ny, j % nx] = np.cos(0.5 * seed_angle)
                q4[i % ny, j % nx] = np.sin(0.5 * seed_angle)
    if ncomp == 2 and not isinstance(c0, (list, tuple)):
        return phi, q1, q4, np.full(shape, 0.5 if c0 is None else c0)
    vals = list(c0) if c0 is not None else [1.0 / ncomp] * (ncomp - 1)
    return (phi, q1, q4) + tuple(np.full(shape, v) for v in vals)


def noise_normal(seed: int, step: int, shape, stream: int = 0) -> np.ndarray:
    """N(0,1) per cell: Box-Muller on two uniforms made from words 2k and
    2k+1 of the Philox4x32-10 block with counter (col / 2, row, step low,
    step high) and key (seed low ^ (0x5eed0000 + stream), seed high); cell
    (row, col) takes pair k = col % 2. Streams (NCGPU_new): 0 .. N - 2 the
    concentration noise of each component (NCGPU draws stream 0 only),
    NOISE_PHI, NOISE_Q1, NOISE_Q4 the phase and orientation noise. u1 = (top 24 bits + 1/2) 2^-24 (never 0),
    u2 = top 24 bits 2^-24; z = sqrt(-2 ln u1) cos(2 pi u2). The library
    draws the same numbers."""
    ny, nx = shape
    ng = (nx + 1) // 2
    g = np.tile(np.arange(ng, dtype=np.uint64), ny)
    r = np.repeat(np.arange(ny, dtype=np.uint64), ng)
    step, seed = int(step), int(seed)
    w = philox4x32_10((g, r, step & 0xFFFFFFFF, step >> 32),
                      ((seed & 0xFFFFFFFF) ^ (0x5EED0000 + stream), seed >> 32))
    w = [(x >> np.uint64(8)).astype(np.float64) for x in w]
    z = []
    for k in range(2):
        u1 = (w[2 * k] + 0.5) * 2.0 ** -24
        u2 = w[2 * k + 1] * 2.0 ** -24
        z.append(np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2))
    out = np.stack(z, axis=-1).reshape(ny, 2 * ng)[:, :nx]
    return out


NOISE_PHI, NOISE_Q1, NOISE_Q4 = 8, 9, 10


def noise_new(seed: int, step: int, shape, nc: int) -> dict:
    """The N(0,1) fields NCGPU_new draws in one step: one per concentration
    field, and for phi, q1 and q4."""
    return {"c": [noise_normal(seed, step, shape, l) for l in range(nc)],
            "phi": noise_normal(seed, step, shape, NOISE_PHI),
            "q1": noise_normal(seed, step, shape, NOISE_Q1),
            "q4": noise_normal(seed, step, shape, NOISE_Q4)}


def _pad(a, bc):
    mode = "wrap" if bc == "PERIODIC" else "symmetric"
    return np.pad(a, 1, mode=mode)


def step(fields, T, p: dict, tdb: Tdb, noise, bc: str = "PERIODIC", noise_scale: float = 1.0,
         variant: str = "NCGPU"):
    """One NCGPU step (helper kernel, then main kernel) on interior arrays
    (phi, q1, q4, c_1 .. c_{N-1}); the last component's fraction is 1 - sum
    c. T an interior array. `bc`: PERIODIC or NEUMANN (zero gradient),
    applied to every field as ghost cells. As the reference, dG/dc is taken
    once per cell (first component up, last one down, :282-286) and used for
    every component; `noise` is the interior N(0,1) field.

    variant "NCGPU_new" (Engines/NCGPU_new.py): dG/dc_l per component (the
    last component down once, then component l up and back, in place, as
    :298-313 mutate their input array), a noise draw per component scaled by
    noise_c, the phase noise sqrt(2 R T M_phi / v_m) noise_phi added after
    the mobility (:186-189), orientation noise sqrt(1e-10 R T / v_m)
    noise_q inside the quaternion brackets (:225-231), eqbar = 0.1 ebar,
    ebar^2 and eqbar^2 as products of the square roots (:78-79), phi clamped
    to [1e-4, 0.9999]; `noise` is noise_new()'s dict."""
    P, Q1, Q4, CC, TT, GL, GS, MC, DF = thermo(fields, T, p, tdb, noise, bc, noise_scale, variant)
    idx = 1.0 / p["dx"]
    if variant == "NCGPU_new":
        ebar2, eqbar2 = p["ebar"] * p["ebar"], p["eqbar"] * p["eqbar"]
        return _update(P, Q1, Q4, CC, TT, GL, GS, MC, DF, p, ebar2, eqbar2, idx, noise=noise,
                       clamp=(0.0001, 0.9999))
    ebar2 = 6.0 * math.sqrt(2.0) * p["S"][1] * p["d"] / p["T_M"][1]
    return _update(P, Q1, Q4, CC, TT, GL, GS, MC, DF, p, ebar2, 0.25 * ebar2, idx)


def thermo(fields, T, p: dict, tdb: Tdb, noise, bc: str = "PERIODIC", noise_scale: float = 1.0,
           variant: str = "NCGPU"):
    """The helper kernel of a step (see `step`): returns the padded fields
    P, Q1, Q4, CC (concentrations), TT (temperature), the interior G_L and
    G_S, and the padded M_c and dF/dc of every concentration field."""
    new = variant == "NCGPU_new"
    phi, q1, q4 = fields[:3]
    cs = list(fields[3:])
    nc = len(cs)
    phases = tdb.phases  # sorted: FCC_A1 (solid), LIQUID
    v_m, D_L, D_S = p["v_m"], p["D_L"], p["D_S"]
    W = p["W"]
    ny, nx = phi.shape
    # helper: thermodynamics per interior cell
    GL = np.empty_like(phi)
    GS = np.empty_like(phi)
    Mcs = [np.empty_like(phi) for _ in range(nc)]
    dFs = [np.empty_like(phi) for _ in range(nc)]
    for i in range(ny):
        for j in range(nx):
            t = T[i, j]
            xs = [c[i, j] for c in cs]
            xs.append(1.0 - sum(xs))
            gl = tdb.gibbs(phases[1], xs, t)
            gs = tdb.gibbs(phases[0], xs, t)
            ph = phi[i, j]
            g = ph * ph * (1 - ph) ** 2
            h = ph ** 3 * (6 * ph * ph - 15 * ph + 10)
            GL[i, j], GS[i, j] = gl, gs
            if new:
                x = list(xs)
                x[nc] -= 1e-7
                for l in range(nc):
                    x[l] += 1e-7
                    dgl = 1e7 * (tdb.gibbs(phases[1], x, t) - gl)
                    dgs = 1e7 * (tdb.gibbs(phases[0], x, t) - gs)
                    Mcs[l][i, j] = v_m * xs[l] * (D_L + h * (D_S - D_L)) / (R_KERNEL * t)
                    nz = p["noise_c"] * math.sqrt(2.0 * R_KERNEL * t / v_m) * noise["c"][l][i, j]
                    dFs[l][i, j] = (dgl + h * (dgs - dgl)) / v_m + (W[l] - W[nc]) * g * t + nz
                    x[l] -= 1e-7
                continue
            xp = list(xs)
            xp[nc] -= 1e-7
            xp[0] += 1e-7
            dgl = 1e7 * (tdb.gibbs(phases[1], xp, t) - gl)
            dgs = 1e7 * (tdb.gibbs(phases[0], xp, t) - gs)
            nz = noise_scale * math.sqrt(2.0 * R_KERNEL * t / v_m) * noise[i, j]
            for l in range(nc):
                Mcs[l][i, j] = v_m * xs[l] * (D_L + h * (D_S - D_L)) / (R_KERNEL * t)
                dFs[l][i, j] = (dgl + h * (dgs - dgl)) / v_m + (W[l] - W[nc]) * g * t + nz
    P, Q1, Q4, TT = (_pad(a, bc) for a in (phi, q1, q4, T))
    CC = [_pad(a, bc) for a in cs]
    MC = [_pad(a, bc) for a in Mcs]
    DF = [_pad(a, bc) for a in dFs]
    return P, Q1, Q4, CC, TT, GL, GS, MC, DF


def _update(P, Q1, Q4, CC, TT, GL, GS, MC, DF, p, ebar2, eqbar2, idx, noise=None,
            clamp=(0.000001, 0.999999)):
    """NComponent_kernel (:37-242) on padded arrays; with `noise` (a
    noise_new() dict) the NCGPU_new kernel's phase and orientation noise."""
    v_m, W, M = p["v_m"], p["W"], p["M"]
    y_e, H, beta, M_qmax, dt = p["y_e"], p["H"], p["beta"], p["M_qmax"], p["dt"]
    nc = len(CC)
    ny, nx = P.shape[0] - 2, P.shape[1] - 2
    out = [np.empty((ny, nx)) for _ in range(3 + nc)]
    for i in range(1, ny + 1):
        for j in range(1, nx + 1):
            ph = P[i, j]
            g = ph * ph * (1 - ph) ** 2
            h = ph ** 3 * (6 * ph * ph - 15 * ph + 10)
            hprime = 30 * g
            gprime = 4 * ph ** 3 - 6 * ph ** 2 + 2 * ph
            dpx = 0.5 * (P[i, j + 1] - P[i, j - 1]) * idx
            dpy = 0.5 * (P[i + 1, j] - P[i - 1, j]) * idx
            dTx = 0.5 * idx * (TT[i, j + 1] - TT[i, j - 1])
            dTy = 0.5 * idx * (TT[i + 1, j] - TT[i - 1, j])
            pxx = (P[i, j + 1] + P[i, j - 1] - 2 * ph) * idx * idx
            pyy = (P[i + 1, j] + P[i - 1, j] - 2 * ph) * idx * idx
            lphi = pxx + pyy
            pxy = 0.25 * (P[i + 1, j + 1] - P[i + 1, j - 1] - P[i - 1, j + 1] + P[i - 1, j - 1]) * idx * idx
            mg2 = max(dpx ** 2 + dpy ** 2, 1e-6)
            mg4 = mg2 * mg2
            mg8 = mg4 * mg4
            a1, a4 = Q1[i, j], Q4[i, j]
            dq1x = 0.5 * idx * (Q1[i, j + 1] - Q1[i, j - 1])
            dq1y = 0.5 * idx * (Q1[i + 1, j] - Q1[i - 1, j])
            dq4x = 0.5 * idx * (Q4[i, j + 1] - Q4[i, j - 1])
            dq4y = 0.5 * idx * (Q4[i + 1, j] - Q4[i - 1, j])
            gxp = idx * math.sqrt((Q1[i, j + 1] - a1) ** 2 + (Q4[i, j + 1] - a4) ** 2)
            gxm = idx * math.sqrt((Q1[i, j - 1] - a1) ** 2 + (Q4[i, j - 1] - a4) ** 2)
            gyp = idx * math.sqrt((Q1[i + 1, j] - a1) ** 2 + (Q4[i + 1, j] - a4) ** 2)
            gym = idx * math.sqrt((Q1[i - 1, j] - a1) ** 2 + (Q4[i - 1, j] - a4) ** 2)
            mgq = 0.5 * (gxp + gxm + gyp + gym)
            gxp, gxm, gyp, gym = (max(v, beta) for v in (gxp, gxm, gyp, gym))
            q2q2 = a1 * a1 - a4 * a4
            qq2 = 2 * a1 * a4
            psx = q2q2 * dpx - qq2 * dpy
            psy = qq2 * dpx + q2q2 * dpy
            psx2, psy2 = psx * psx, psy * psy
            psx3, psy3 = psx2 * psx, psy2 * psy
            psx4, psy4 = psx2 * psx2, psy2 * psy2
            dq2q2dx = 2 * a1 * dq1x - 2 * a4 * dq4x
            dqq2dx = 2 * a4 * dq1x + 2 * a1 * dq4x
            dq2q2dy = 2 * a1 * dq1y - 2 * a4 * dq4y
            dqq2dy = 2 * a4 * dq1y + 2 * a1 * dq4y
            dpsxdx = dq2q2dx * dpx + q2q2 * pxx - dqq2dx * dpy - qq2 * pxy
            dpsxdy = dq2q2dy * dpx + q2q2 * pxy - dqq2dy * dpy - qq2 * pyy
            dpsydx = dq2q2dx * dpy + q2q2 * pxy + dqq2dx * dpx + qq2 * pxx
            dpsydy = dq2q2dy * dpy + q2q2 * pyy + dqq2dy * dpx + qq2 * pxy
            t = TT[i, j]
            s4 = psx4 + psy4
            tx = dTx * ((2 * psx3 * q2q2 + 2 * psy3 * qq2) / mg2 - dpx * s4 / mg4)
            tx += t * (6 * psx2 * dpsxdx * q2q2 + 2 * psx3 * dq2q2dx + 6 * psy2 * dpsydx * qq2
                       + 2 * psy3 * dqq2dx) / mg2
            tx -= t * (2 * psx3 * q2q2 + 2 * psy3 * qq2) * (2 * dpx * pxx + 2 * dpy * pxy) / mg4
            tx -= t * (pxx * s4 + dpx * (4 * psx3 * dpsxdx + 4 * psy3 * dpsydx)) / mg4
            tx += t * (dpx * s4 * (4 * dpx ** 3 * pxx + 4 * dpx * pxx * dpy ** 2
                                   + 4 * dpy * pxy * dpx ** 2 + 4 * dpy ** 3 * pxy)) / mg8
            tx *= 4 * y_e * ebar2
            ty = dTy * ((-2 * psx3 * qq2 + 2 * psy3 * q2q2) / mg2 - dpy * s4 / mg4)
            ty += t * (-6 * psx2 * dpsxdy * qq2 - 2 * psx3 * dqq2dy + 6 * psy2 * dpsydy * q2q2
                       + 2 * psy3 * dq2q2dy) / mg2
            ty -= t * (-2 * psx3 * qq2 + 2 * psy3 * q2q2) * (2 * dpx * pxy + 2 * dpy * pyy) / mg4
            ty -= t * (pyy * s4 + dpy * (4 * psx3 * dpsxdy + 4 * psy3 * dpsydy)) / mg4
            ty += t * (dpy * s4 * (4 * dpx ** 3 * pxy + 4 * dpx * pxy * dpy ** 2
                                   + 4 * dpy * pyy * dpx ** 2 + 4 * dpy ** 3 * pyy)) / mg8
            ty *= 4 * y_e * ebar2
            cW, c_N, M_phi = 0.0, 1.0, 0.0
            for l in range(nc):
                cl = CC[l][i, j]
                cW += cl * W[l]
                c_N -= cl
                M_phi += cl * M[l]
            cW += c_N * W[nc]
            M_phi += c_N * M[nc]
            M_q = M_qmax + (1e-6 - M_qmax) * h
            dphidt = ebar2 * (1 - 3 * y_e) * (t * lphi + dTx * dpx + dTy * dpy)
            dphidt += tx + ty
            dphidt -= hprime * (GS[i - 1, j - 1] - GL[i - 1, j - 1]) / v_m
            dphidt -= gprime * t * cW
            dphidt -= 4 * H * t * ph * mgq
            dphidt *= M_phi
            nq1 = nq4 = 0.0
            if noise is not None:
                dphidt += (math.sqrt(2.0 * R_KERNEL * t * M_phi / v_m) * noise["phi"][i - 1, j - 1]
                           * p["noise_phi"])
                qa = p["noise_q"] * math.sqrt(0.0000000001 * R_KERNEL * t / v_m)
                nq1 = qa * noise["q1"][i - 1, j - 1]
                nq4 = qa * noise["q4"][i - 1, j - 1]

            def divagradb(a, axp, axm, ayp, aym, b, bxp, bxm, byp, bym):
                return 0.5 * idx * idx * ((axp + a) * (bxp - b) - (a + axm) * (b - bxm)
                                          + (ayp + a) * (byp - b) - (a + aym) * (b - bym))

            def nb5(A):
                return A[i, j], A[i, j + 1], A[i, j - 1], A[i + 1, j], A[i - 1, j]

            dcs = []
            for l in range(nc):
                m, mxp, mxm, myp, mym = nb5(MC[l])
                dc = divagradb(m, mxp, mxm, myp, mym, *nb5(DF[l]))
                for k in range(nc):
                    c0_, cxp, cxm, cyp, cym = nb5(CC[k])
                    dc -= divagradb(m * c0_, mxp * cxp, mxm * cxm, myp * cyp, mym * cym,
                                    *nb5(DF[k]))
                dcs.append(dc)
            Dq = 2 * H * t * ph * ph
            Dxp = 2 * H * TT[i, j + 1] * P[i, j + 1] ** 2
            Dxm = 2 * H * TT[i, j - 1] * P[i, j - 1] ** 2
            Dyp = 2 * H * TT[i + 1, j] * P[i + 1, j] ** 2
            Dym = 2 * H * TT[i - 1, j] * P[i - 1, j] ** 2

            def fori(q, qxp, qxm, qyp, qym):
                return 0.5 * idx * idx * ((Dq + Dxp) * (qxp - q) / gxp - (Dq + Dxm) * (q - qxm) / gxm
                                          + (Dq + Dyp) * (qyp - q) / gyp - (Dq + Dym) * (q - qym) / gym)

            f1 = fori(a1, Q1[i, j + 1], Q1[i, j - 1], Q1[i + 1, j], Q1[i - 1, j])
            f4 = fori(a4, Q4[i, j + 1], Q4[i, j - 1], Q4[i + 1, j], Q4[i - 1, j])
            lq1 = (Q1[i, j + 1] + Q1[i, j - 1] + Q1[i + 1, j] + Q1[i - 1, j] - 4 * a1) * idx * idx
            lq4 = (Q4[i, j + 1] + Q4[i, j - 1] + Q4[i + 1, j] + Q4[i - 1, j] - 4 * a4) * idx * idx
            if noise is None:
                dq1 = M_q * ((1 - a1 * a1) * (f1 + lq1 * eqbar2) - a1 * a4 * (f4 + lq4 * eqbar2))
                dq4 = M_q * ((1 - a4 * a4) * (f4 + lq4 * eqbar2) - a1 * a4 * (f1 + lq1 * eqbar2))
            else:
                b1 = f1 + lq1 * eqbar2 - 0.0 + nq1
                b4 = f4 + lq4 * eqbar2 - 0.0 + nq4
                dq1 = M_q * ((1 - a1 * a1) * b1 - a1 * a4 * b4)
                dq4 = M_q * ((1 - a4 * a4) * b4 - a1 * a4 * b1)
            pn = min(max(ph + dt * dphidt, clamp[0]), clamp[1])
            n1, n4 = a1 + dt * dq1, a4 + dt * dq4
            rn = math.sqrt(n1 * n1 + n4 * n4)
            out[0][i - 1, j - 1] = pn
            out[1][i - 1, j - 1] = n1 / rn
            out[2][i - 1, j - 1] = n4 / rn
            for l in range(nc):
                out[3 + l][i - 1, j - 1] = CC[l][i, j] + dt * dcs[l]
    return out


def run(fields, T, steps, p, tdb, seed=0, bc="PERIODIC", noise_scale=1.0, step0=0,
        variant="NCGPU", dT_step=0.0):
    """`steps` steps from absolute step index step0. dT_step: the temperature
    rise per step of a LINEAR_GRADIENT temperature with dT/dt (dTdt * dt):
    every step reads T, then T += dT_step on every cell
    (Simulation.simulate, simulation.py:262-266, with
    update_thermal_gradient_2D_kernel, ppf_gpu_utils.py:326-334)."""
    f = [np.array(a, dtype=np.float64) for a in fields]
    T = np.array(T, dtype=np.float64)
    for s in range(steps):
        if variant == "NCGPU_new":
            nz = noise_new(seed, step0 + s, f[0].shape, len(f) - 3)
        else:
            nz = noise_normal(seed, step0 + s, f[0].shape) if noise_scale else np.zeros(f[0].shape)
        f = step(f, T, p, tdb, nz, bc, noise_scale, variant)
        if dT_step:
            T += dT_step
    return f
