"""Float32 emulation of the NCGPU update kernel on the CPU (test
infrastructure: only tests/ use it).

The CUDA kernel (pyphasefield_gb300/csrc/ncgpu.cu, ncgpu_kernel) evaluates
the thermodynamics in float64 and the update in the field precision; in
float32 its thresholds (|grad q| clamped at beta, phi clamped) can fall the
other way than in float64 for single cells. This module repeats the float32
update, expression by expression, with numpy float32 arrays (the anisotropy
on the unit vectors grad phi / |grad phi| as the kernel evaluates it), on
top of the float64 thermodynamics of oracle.ncgpu_ref, so that the float32
tolerances of the GPU tests can be set from a CPU run of the same
arithmetic. Reference: Engines/NCGPU.py:37-242, Engines/NCGPU_new.py:38-252.
"""
from __future__ import annotations

import numpy as np

from . import ncgpu_ref as N

F = np.float32

def _c(A):
    return A[1:-1, 1:-1]


def _xp(A):
    return A[1:-1, 2:]


def _xm(A):
    return A[1:-1, :-2]


def _yp(A):
    return A[2:, 1:-1]


def _ym(A):
    return A[:-2, 1:-1]


def _face(idx, beta, d1, d4):
    """|grad q| across a face and the reciprocal of its value clamped at
    beta, from one reciprocal square root (s = 0 takes 1 / beta)."""
    sq = d1 * d1 + d4 * d4
    r = np.where(sq > 0, F(1) / np.sqrt(np.where(sq > 0, sq, F(1))), F(0)).astype(F)
    g = idx * (sq * r)
    ig = np.where(g < beta, F(1) / beta, (F(1) / idx) * r).astype(F)
    return g, ig


def main_kernel32(P, Q1, Q4, CC, TT, GL, GS, MC, DF, p, ebar2, eqbar2, variant, noise):
    """One update on padded float32 arrays (GL, GS interior); returns the
    interior fields, in the kernel's order of operations."""
    c, xp, xm, yp, ym = _c, _xp, _xm, _yp, _ym
    idx = F(1.0 / p["dx"])
    ph = c(P)
    gg = ph * ph * (F(1) - ph) * (F(1) - ph)
    h = ph * ph * ph * (F(6) * ph * ph - F(15) * ph + F(10))
    hprime = F(30) * gg
    gprime = F(4) * ph * ph * ph - F(6) * ph * ph + F(2) * ph
    dpx = F(0.5) * (xp(P) - xm(P)) * idx
    dpy = F(0.5) * (yp(P) - ym(P)) * idx
    t = c(TT)
    dTx = F(0.5) * idx * (xp(TT) - xm(TT))
    dTy = F(0.5) * idx * (yp(TT) - ym(TT))
    pxx = (xp(P) + xm(P) - F(2) * ph) * idx * idx
    pyy = (yp(P) + ym(P) - F(2) * ph) * idx * idx
    lphi = pxx + pyy
    pxy = F(0.25) * (P[2:, 2:] - P[2:, :-2] - P[:-2, 2:] + P[:-2, :-2]) * idx * idx
    mg2 = np.maximum(dpx * dpx + dpy * dpy, F(1e-6))
    a1, a4 = c(Q1), c(Q4)
    dq1x = F(0.5) * idx * (xp(Q1) - xm(Q1))
    dq1y = F(0.5) * idx * (yp(Q1) - ym(Q1))
    dq4x = F(0.5) * idx * (xp(Q4) - xm(Q4))
    dq4y = F(0.5) * idx * (yp(Q4) - ym(Q4))
    beta = F(p["beta"])
    gxp, igxp = _face(idx, beta, xp(Q1) - a1, xp(Q4) - a4)
    gxm, igxm = _face(idx, beta, xm(Q1) - a1, xm(Q4) - a4)
    gyp, igyp = _face(idx, beta, yp(Q1) - a1, yp(Q4) - a4)
    gym, igym = _face(idx, beta, ym(Q1) - a1, ym(Q4) - a4)
    mgq = F(0.5) * (gxp + gxm + gyp + gym)
    # anisotropy on the unit vectors u = grad phi / m, s = psi / m
    q2q2, qq2 = a1 * a1 - a4 * a4, F(2) * a1 * a4
    im = F(1) / np.sqrt(mg2)
    m = mg2 * im
    ux, uy = dpx * im, dpy * im
    sx = (q2q2 * dpx - qq2 * dpy) * im
    sy = (qq2 * dpx + q2q2 * dpy) * im
    sx2, sy2 = sx * sx, sy * sy
    sx3, sy3 = sx2 * sx, sy2 * sy
    s4 = sx2 * sx2 + sy2 * sy2
    dq2q2dx = F(2) * a1 * dq1x - F(2) * a4 * dq4x
    dqq2dx = F(2) * a4 * dq1x + F(2) * a1 * dq4x
    dq2q2dy = F(2) * a1 * dq1y - F(2) * a4 * dq4y
    dqq2dy = F(2) * a4 * dq1y + F(2) * a1 * dq4y
    dpsxdx = dq2q2dx * dpx + q2q2 * pxx - dqq2dx * dpy - qq2 * pxy
    dpsxdy = dq2q2dy * dpx + q2q2 * pxy - dqq2dy * dpy - qq2 * pyy
    dpsydx = dq2q2dx * dpy + q2q2 * pxy + dqq2dx * dpx + qq2 * pxx
    dpsydy = dq2q2dy * dpy + q2q2 * pyy + dqq2dy * dpx + qq2 * pxy
    ux2, uy2 = ux * ux, uy * uy
    ye, eb2 = F(p["y_e"]), F(ebar2)
    tx = dTx * m * (F(2) * sx3 * q2q2 + F(2) * sy3 * qq2 - ux * s4)
    tx += t * (F(6) * sx2 * dpsxdx * q2q2 + F(2) * sx3 * m * dq2q2dx
               + F(6) * sy2 * dpsydx * qq2 + F(2) * sy3 * m * dqq2dx)
    tx -= t * (F(2) * sx3 * q2q2 + F(2) * sy3 * qq2) * (F(2) * ux * pxx + F(2) * uy * pxy)
    tx -= t * (pxx * s4 + ux * (F(4) * sx3 * dpsxdx + F(4) * sy3 * dpsydx))
    tx += t * (ux * s4 * (F(4) * ux2 * ux * pxx + F(4) * ux * pxx * uy2
                          + F(4) * uy * pxy * ux2 + F(4) * uy2 * uy * pxy))
    tx *= F(4) * ye * eb2
    ty = dTy * m * (-F(2) * sx3 * qq2 + F(2) * sy3 * q2q2 - uy * s4)
    ty += t * (-F(6) * sx2 * dpsxdy * qq2 - F(2) * sx3 * m * dqq2dy
               + F(6) * sy2 * dpsydy * q2q2 + F(2) * sy3 * m * dq2q2dy)
    ty -= t * (-F(2) * sx3 * qq2 + F(2) * sy3 * q2q2) * (F(2) * ux * pxy + F(2) * uy * pyy)
    ty -= t * (pyy * s4 + uy * (F(4) * sx3 * dpsxdy + F(4) * sy3 * dpsydy))
    ty += t * (uy * s4 * (F(4) * ux2 * ux * pxy + F(4) * ux * pxy * uy2
                          + F(4) * uy * pyy * ux2 + F(4) * uy2 * uy * pyy))
    ty *= F(4) * ye * eb2
    nc = len(CC)
    W = [F(w) for w in p["W"]]
    M = [F(x) for x in p["M"]]
    cW, Mphi, cN = np.zeros_like(ph), np.zeros_like(ph), np.ones_like(ph)
    for l in range(nc):
        cl = c(CC[l])
        cW += cl * W[l]
        Mphi += cl * M[l]
        cN -= cl
    cW += cN * W[nc]
    Mphi += cN * M[nc]
    Mq = F(p["M_qmax"]) + (F(1e-6) - F(p["M_qmax"])) * h
    v_m, H = F(p["v_m"]), F(p["H"])
    dphidt = eb2 * (F(1) - F(3) * ye) * (t * lphi + dTx * dpx + dTy * dpy)
    dphidt += tx + ty
    dphidt -= hprime * (GS - GL) / v_m
    dphidt -= gprime * t * cW
    dphidt -= F(4) * H * t * ph * mgq
    dphidt *= Mphi
    nq1 = nq4 = F(0)
    if variant:
        dphidt += np.sqrt(F(2) * F(8.314) * t * Mphi / v_m) * noise["phi"].astype(F) * \
            F(p["noise_phi"])
        qa = F(p["noise_q"]) * np.sqrt(F(1e-10) * F(8.314) * t / v_m)
        nq1 = qa * noise["q1"].astype(F)
        nq4 = qa * noise["q4"].astype(F)

    def divagradb(a, axp, axm, ayp, aym, b, bxp, bxm, byp, bym):
        return F(0.5) * idx * idx * ((axp + a) * (bxp - b) - (a + axm) * (b - bxm)
                                     + (ayp + a) * (byp - b) - (a + aym) * (b - bym))

    def nb(A):
        return c(A), xp(A), xm(A), yp(A), ym(A)

    dcs = []
    for l in range(nc):
        m0, mxp, mxm, myp, mym = nb(MC[l])
        d = divagradb(m0, mxp, mxm, myp, mym, *nb(DF[l]))
        for k in range(nc):
            c0, cxp, cxm, cyp, cym = nb(CC[k])
            d -= divagradb(m0 * c0, mxp * cxp, mxm * cxm, myp * cyp, mym * cym, *nb(DF[k]))
        dcs.append(d)
    twoH = F(2) * H
    Dq = twoH * t * ph * ph
    rxp = (Dq + twoH * xp(TT) * xp(P) * xp(P)) * igxp
    rxm = (Dq + twoH * xm(TT) * xm(P) * xm(P)) * igxm
    ryp = (Dq + twoH * yp(TT) * yp(P) * yp(P)) * igyp
    rym = (Dq + twoH * ym(TT) * ym(P) * ym(P)) * igym

    def fori(q, A):
        return F(0.5) * idx * idx * (rxp * (xp(A) - q) - rxm * (q - xm(A))
                                     + ryp * (yp(A) - q) - rym * (q - ym(A)))

    f1, f4 = fori(a1, Q1), fori(a4, Q4)
    lq1 = (xp(Q1) + xm(Q1) + yp(Q1) + ym(Q1) - F(4) * a1) * idx * idx
    lq4 = (xp(Q4) + xm(Q4) + yp(Q4) + ym(Q4) - F(4) * a4) * idx * idx
    eq2 = F(eqbar2)
    b1 = f1 + lq1 * eq2 + nq1
    b4 = f4 + lq4 * eq2 + nq4
    dq1 = Mq * ((F(1) - a1 * a1) * b1 - a1 * a4 * b4)
    dq4 = Mq * ((F(1) - a4 * a4) * b4 - a1 * a4 * b1)
    dt = F(p["dt"])
    lo, hi = (F(1e-4), F(0.9999)) if variant else (F(1e-6), F(0.999999))
    pn = np.clip(ph + dt * dphidt, lo, hi)
    n1, n4 = a1 + dt * dq1, a4 + dt * dq4
    irn = F(1) / np.sqrt(n1 * n1 + n4 * n4)
    return [pn, n1 * irn, n4 * irn] + [c(CC[l]) + dt * dcs[l] for l in range(nc)]


def run(fields, T, steps, p, tdb, seed, bc, variant):
    """`steps` steps in float32 from interior float64 fields; p from
    ncgpu_ref.tdb_params(..., variant=variant). The thermodynamics of each
    step are ncgpu_ref.thermo's (float64, as on the GPU), rounded to
    float32 as the kernel stores them."""
    new = variant == "NCGPU_new"
    if new:
        ebar2, eqbar2 = p["ebar"] * p["ebar"], p["eqbar"] * p["eqbar"]
    else:
        ebar2 = p["ebar"] * p["ebar"]
        eqbar2 = 0.25 * ebar2
    f = [np.asarray(a, np.float64).astype(F) for a in fields]
    for s in range(steps):
        shape = f[0].shape
        nz = N.noise_new(seed, s, shape, len(f) - 3) if new else N.noise_normal(seed, s, shape)
        P, Q1, Q4, CC, TT, GL, GS, MC, DF = N.thermo([x.astype(np.float64) for x in f], T, p,
                                                     tdb, nz, bc, 1.0, variant)
        f = main_kernel32(_f32(P), _f32(Q1), _f32(Q4), [_f32(a) for a in CC], _f32(TT), _f32(GL),
                          _f32(GS), [_f32(a) for a in MC], [_f32(a) for a in DF], p, ebar2,
                          eqbar2, new, nz if new else None)
    return [np.asarray(a, np.float64) for a in f]


def _f32(a):
    return np.asarray(a).astype(F)
