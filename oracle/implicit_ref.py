"""CPU restatement of pyphasefield's implicit and Crank-Nicolson diffusion
engines (test infrastructure: only tests/ and bench.py's CPU legs use it).

Reference: Engines/Diffusion.py
  diffusion_matrix_1d / _2d / _3d      :18-196   periodic matrices
  engine_ImplicitDiffusion{1,2,3}D     :210-306  np.linalg.solve of the full system
  engine_CrankNicolsonDiffusion{1,2,3}D :309-411 explicit half step, then solve
  engine_ImplicitDiffusion{2,3}D_ADI   :413-510  1-D solves axis by axis
  engine_CrankNicolsonDiffusion{2,3}D_ADI :512-633 explicit half + 1-D solve per axis
  the *_GMRES twins approximate the same systems with scipy's gmres.

Every function here works on the interior cells with periodic wrap, which is
what the reference's matrices encode ("Matrix shows periodic boundary
conditions!", :23). The reference itself hands the padded Field.data
(interior + 2 ghost cells per axis, field.py:6-20) to matrices sized for the
interior, reads an undefined global ``self`` (:206 and every engine) and an
undefined ``dim`` in Diffusion.simulation_loop (:671-720); applied to the
interior array with the user_data it means, its engine functions run as
written, and tests/golden/make_golden.py pins this module to them.

The reference's matrix builders overwrite rather than add when an axis has
fewer than 3 cells (both neighbours of a cell are then the same cell); the
restatement, like the library, requires >= 3 cells per solved axis.
"""
from __future__ import annotations

import numpy as np


def periodic_matrix_1d(n: int, center: float, neighbor: float) -> np.ndarray:
    """Dense periodic tridiagonal matrix (diffusion_matrix_1d, :18-64)."""
    m = np.zeros((n, n))
    idx = np.arange(n)
    m[idx, idx] = center
    m[idx, (idx - 1) % n] = neighbor
    m[idx, (idx + 1) % n] = neighbor
    return m


def periodic_matrix_nd(shape, center: float, neighbor: float) -> np.ndarray:
    """Dense periodic 2d+1 / 4d... point matrix on C-order flattened cells
    (diffusion_matrix_2d :66-126, diffusion_matrix_3d :128-196)."""
    n = int(np.prod(shape))
    m = np.zeros((n, n))
    cells = np.arange(n).reshape(shape)
    m[cells.ravel(), cells.ravel()] = center
    for ax in range(len(shape)):
        for sh in (1, -1):
            m[cells.ravel(), np.roll(cells, sh, ax).ravel()] = neighbor
    return m


def explicit_half(c: np.ndarray, alpha: float, axis: int) -> np.ndarray:
    """(1 - 2 alpha) c + alpha (c[i-1] + c[i+1]) along one axis, periodic
    (the np.roll lines of the Crank-Nicolson ADI engines, :527, :580)."""
    return (1 - 2 * alpha) * c + alpha * (np.roll(c, 1, axis) + np.roll(c, -1, axis))


def explicit_full(c: np.ndarray, alpha: float) -> np.ndarray:
    """(1 - 2 d alpha) c + alpha * sum of the 2d neighbours (:322, :357, :391)."""
    out = (1 - 2 * c.ndim * alpha) * c
    for ax in range(c.ndim):
        out = out + alpha * (np.roll(c, 1, ax) + np.roll(c, -1, ax))
    return out


def line_solve(c: np.ndarray, alpha: float, axis: int) -> np.ndarray:
    """Solve the periodic 1-D system (1+2a) x_i - a (x_{i-1} + x_{i+1}) = c_i
    along `axis` for every line (the np.dot(inv, line) loops of the ADI
    engines, :428-431, :474-482)."""
    n = c.shape[axis]
    if n < 3:
        raise ValueError("periodic line solves need >= 3 cells per axis")
    m = periodic_matrix_1d(n, 1 + 2 * alpha, -alpha)
    moved = np.moveaxis(np.asarray(c, dtype=np.float64), axis, 0)
    x = np.linalg.solve(m, moved.reshape(n, -1)).reshape(moved.shape)
    return np.moveaxis(x, 0, axis)


def full_solve_dense(rhs: np.ndarray, alpha: float) -> np.ndarray:
    """Solve the full periodic system by a dense factorisation, as the
    reference does (np.linalg.solve of diffusion_matrix_nd, :253-256)."""
    if min(rhs.shape) < 3:
        raise ValueError("periodic solves need >= 3 cells per axis")
    m = periodic_matrix_nd(rhs.shape, 1 + 2 * rhs.ndim * alpha, -alpha)
    return np.linalg.solve(m, rhs.ravel()).reshape(rhs.shape)


def full_solve_fft(rhs: np.ndarray, alpha: float) -> np.ndarray:
    """The same solve by the discrete Fourier transform (the periodic matrix
    is circulant: eigenvalue 1 + 2 alpha sum(1 - cos theta) per mode); used
    for grids too large for the dense matrix, checked against it."""
    lam = np.ones(rhs.shape)
    for ax, n in enumerate(rhs.shape):
        theta = 2 * np.pi * np.arange(n) / n
        shape = [1] * rhs.ndim
        shape[ax] = n
        lam = lam + 2 * alpha * (1 - np.cos(theta)).reshape(shape)
    return np.real(np.fft.ifftn(np.fft.fftn(rhs) / lam))


def implicit_step(c: np.ndarray, D: float, dt: float, dx: float, adi: bool,
                  dense_limit: int = 4096) -> np.ndarray:
    """One step of the implicit engines (:210-306, :413-510)."""
    c = np.asarray(c, dtype=np.float64)
    alpha = D * dt / dx ** 2
    if c.ndim == 1:
        return line_solve(c, alpha, 0)
    if adi:
        # x (last axis) first, then y, then z (:428-431, :474-482)
        for ax in reversed(range(c.ndim)):
            c = line_solve(c, alpha, ax)
        return c
    if c.size <= dense_limit:
        return full_solve_dense(c, alpha)
    return full_solve_fft(c, alpha)


def crank_nicolson_step(c: np.ndarray, D: float, dt: float, dx: float, adi: bool,
                        dense_limit: int = 4096) -> np.ndarray:
    """One step of the Crank-Nicolson engines (:309-411, :512-633)."""
    c = np.asarray(c, dtype=np.float64)
    alpha = 0.5 * D * dt / dx ** 2
    if c.ndim == 1:
        return line_solve(explicit_half(c, alpha, 0), alpha, 0)
    if adi:
        if c.ndim == 2:
            # explicit along axis 0, solve along axis 0; explicit along
            # axis 1, solve along axis 1 (:527-533)
            c = line_solve(explicit_half(c, alpha, 0), alpha, 0)
            return line_solve(explicit_half(c, alpha, 1), alpha, 1)
        # explicit 0 / solve 1, explicit 1 / solve 0, explicit 2 / solve 2
        # (:580-591)
        c = line_solve(explicit_half(c, alpha, 0), alpha, 1)
        c = line_solve(explicit_half(c, alpha, 1), alpha, 0)
        return line_solve(explicit_half(c, alpha, 2), alpha, 2)
    rhs = explicit_full(c, alpha)
    if c.size <= dense_limit:
        return full_solve_dense(rhs, alpha)
    return full_solve_fft(rhs, alpha)


def step(c, solver: str, D: float, dt: float, dx: float, adi: bool) -> np.ndarray:
    if solver == "implicit":
        return implicit_step(c, D, dt, dx, adi)
    if solver == "crank-nicolson":
        return crank_nicolson_step(c, D, dt, dx, adi)
    raise ValueError(solver)


def run(c0, steps: int, solver: str, D: float, dt: float, dx: float, adi: bool) -> np.ndarray:
    c = np.asarray(c0, dtype=np.float64)
    for _ in range(steps):
        c = step(c, solver, D, dt, dx, adi)
    return c


# ---------------------------------------------------------------------------
# The library's solution methods, restated in float64 for the CPU tests of
# their algebra (the kernels run them in float or double on the GPU).

def recurrence_root(alpha: float) -> float:
    """r in (0, 1) with alpha r^2 - (1 + 2 alpha) r + alpha = 0, so that the
    periodic operator factors as (alpha / r)(I - r S)(I - r S^-1), S the
    cyclic shift. Written without cancellation for small alpha."""
    return 2 * alpha / (1 + 2 * alpha + np.sqrt(1 + 4 * alpha))


def line_solve_segmented(d: np.ndarray, alpha: float, seg: int) -> np.ndarray:
    """Solve one periodic line the way the line kernels do: two first-order
    cyclic recurrences, each split into segments whose local sums are joined
    by a short carry pass."""
    n = d.size
    r = recurrence_root(alpha)
    dk = d * (r / alpha)
    starts = list(range(0, n, seg))
    F, Bu = [], []
    for p in starts:
        u, bu, pw = 0.0, 0.0, 1.0
        for i in range(p, min(n, p + seg)):
            u = dk[i] + r * u
            bu += pw * u
            pw *= r
        F.append(u)
        Bu.append(bu)
    lens = [min(n, p + seg) - p for p in starts]
    R = [r ** L for L in lens]
    G = [r * (1 - r ** (2 * L)) / (1 - r * r) for L in lens]
    rn = r ** n
    y = 0.0
    for f, rs in zip(F, R):
        y = f + rs * y
    yprev = y / (1 - rn)
    yin, bv = [], []
    for f, b, rs, g in zip(F, Bu, R, G):
        yin.append(yprev)
        bv.append(b + yprev * g)
        yprev = f + rs * yprev
    x = 0.0
    for b, rs in zip(reversed(bv), reversed(R)):
        x = b + rs * x
    xnext = x / (1 - rn)
    xin = [0.0] * len(starts)
    for s in reversed(range(len(starts))):
        xin[s] = xnext
        xnext = bv[s] + R[s] * xnext
    out = np.empty(n)
    for s, p in enumerate(starts):
        q = min(n, p + seg)
        ys = []
        yv = yin[s]
        for i in range(p, q):
            yv = dk[i] + r * yv
            ys.append(yv)
        xv = xin[s]
        for i in reversed(range(p, q)):
            xv = ys[i - p] + r * xv
            out[i] = xv
    return out


def chebyshev_plan(alpha: float, ndim: int, tol: float):
    """Iteration count and weights of the Chebyshev semi-iteration the
    library runs for the full (non-ADI) systems: spectrum of
    A = (1 + 2 d a) I - a sum(S + S^-1) in [1, 1 + 4 d a]; Richardson
    weight gamma = 2 / (lmax + lmin); contraction rho = (lmax - lmin) /
    (lmax + lmin); omega_1 = 1, omega_2 = 2 / (2 - rho^2),
    omega_{k+1} = 1 / (1 - rho^2 omega_k / 4) (Golub and Van Loan, Matrix
    Computations, the Chebyshev semi-iterative method). The count makes the
    bound 2 / T_K(1 / rho) on the error, relative to the field, at most tol
    / (8 d a)."""
    lmax = 1 + 4 * ndim * alpha
    gamma = 2 / (lmax + 1)
    rho = (lmax - 1) / (lmax + 1)
    if rho <= 0:
        return 0, gamma, rho, []
    need = 2 * max(1.0, 8 * ndim * alpha) / tol
    k = int(np.ceil(np.arccosh(need) / np.arccosh(1 / rho)))
    k = max(k, 1)
    om = [1.0]
    if k >= 2:
        om.append(2 / (2 - rho * rho))
    while len(om) < k:
        om.append(1 / (1 - rho * rho * om[-1] / 4))
    return k, gamma, rho, om


def apply_operator(y: np.ndarray, alpha: float) -> np.ndarray:
    out = (1 + 2 * y.ndim * alpha) * y
    for ax in range(y.ndim):
        out = out - alpha * (np.roll(y, 1, ax) + np.roll(y, -1, ax))
    return out


def chebyshev_solve(rhs: np.ndarray, x0: np.ndarray, alpha: float, tol: float) -> np.ndarray:
    k, gamma, rho, om = chebyshev_plan(alpha, rhs.ndim, tol)
    prev, cur = None, np.array(x0, dtype=np.float64)
    for j in range(k):
        nxt = cur + gamma * (rhs - apply_operator(cur, alpha))
        if prev is not None:
            nxt = prev + om[j] * (nxt - prev)
        prev, cur = cur, nxt
    return cur


# ---------------------------------------------------------------------------
# Allen-Cahn ("CahnAllen") and Cahn-Hilliard implicit engines
# (Engines/CahnAllen.py:137-280, Engines/CahnHilliard.py:148-341): periodic
# systems whose diagonal varies per cell.

def var_line_solve(b: np.ndarray, diag: np.ndarray, alpha: float, axis: int) -> np.ndarray:
    """Solve diag_i x_i - alpha (x_{i-1} + x_{i+1}) = b_i, periodic, along
    `axis` for every line; diag has b's shape, or is 1-D (the same diagonal
    for every line, indexed by the position along the line)."""
    n = b.shape[axis]
    if n < 3:
        raise ValueError("periodic line solves need >= 3 cells per axis")
    bm = np.moveaxis(np.asarray(b, dtype=np.float64), axis, 0)
    flat_b = bm.reshape(n, -1)
    if np.ndim(diag) == 1:
        m = periodic_matrix_1d(n, 0.0, -alpha)
        m[np.arange(n), np.arange(n)] = diag
        x = np.linalg.solve(m, flat_b)
    else:
        dm = np.moveaxis(np.asarray(diag, dtype=np.float64), axis, 0).reshape(n, -1)
        x = np.empty_like(flat_b)
        base = periodic_matrix_1d(n, 0.0, -alpha)
        for j in range(flat_b.shape[1]):
            m = base.copy()
            m[np.arange(n), np.arange(n)] = dm[:, j]
            x[:, j] = np.linalg.solve(m, flat_b[:, j])
    return np.moveaxis(x.reshape(bm.shape), 0, axis)


def well_slope(phi):
    """4 phi^2 - 6 phi + 2: the double well's g'(phi) / phi."""
    return 4.0 * phi * phi - 6.0 * phi + 2.0


def allen_cahn_implicit_step(phi, solver: str, M: float, W: float, eps: float, dt: float,
                             dx: float, adi: bool, gmres: bool) -> np.ndarray:
    """One step of CahnAllen.simulation_loop for the non-explicit solvers
    (CahnAllen.py:325-361), each branch restating the engine function it
    calls. Branches the reference leaves empty (Crank-Nicolson in 1-D and
    3-D, IMEX beyond 1-D) return the field unchanged, as it does."""
    phi = np.asarray(phi, dtype=np.float64)
    a = M * dt * eps ** 2 / dx ** 2
    nd = phi.ndim
    if solver == "implicit":
        if nd == 1:  # engine_CahnAllenImplicit1D[_GMRES] :137-162
            return var_line_solve(phi, 1 + 2 * a + 16 * W * M * dt * well_slope(phi), a, 0)
        if nd == 2:
            if gmres and not adi:  # engine_CahnAllenImplicit2D_GMRES :163-175
                diag = 1 + 4 * a + 16 * W * M * dt * well_slope(phi)
                m = periodic_matrix_nd(phi.shape, 0.0, -a)
                m[np.arange(phi.size), np.arange(phi.size)] = diag.ravel()
                return np.linalg.solve(m, phi.ravel()).reshape(phi.shape)
            # engine_CahnAllenImplicit2D_ADI[_GMRES] :176-186, :209-224: rows, then columns,
            # each with the source term of the field as it stands
            phi = var_line_solve(phi, 1 + 2 * a + 8 * W * M * dt * well_slope(phi), a, 1)
            return var_line_solve(phi, 1 + 2 * a + 8 * W * M * dt * well_slope(phi), a, 0)
        # engine_CahnAllenImplicit3D_ADI :225-251: np.fill_diagonal takes the first
        # n entries of the flattened 3-D source term, so every line of an axis
        # shares the diagonal 1 + 2a + s.flat[:n]
        s = (16 * W * M * dt * well_slope(phi) / 3).ravel()
        for ax in (2, 1, 0):
            phi = var_line_solve(phi, 1 + 2 * a + s[:phi.shape[ax]], a, ax)
        return phi
    if solver == "imex":
        if nd != 1:
            return phi
        # engine_CahnAllenIMEX1D :252-267 (its -2 phi term as written)
        rhs = phi - 16 * W * M * dt * (4 * phi ** 3 - 6 * phi ** 2 - 2 * phi)
        return line_solve(rhs, a, 0)
    if solver == "crank-nicolson":
        if nd != 2:
            return phi
        # engine_CahnAllenCrankNicolson2D_ADI :187-208: explicit half along
        # axis 1, rows; explicit half along axis 0, columns; the source term
        # keeps the full dt
        h = 0.5 * a
        phi = explicit_half(phi, h, 1)
        phi = var_line_solve(phi, 1 + 2 * h + 8 * W * M * dt * well_slope(phi), h, 1)
        phi = explicit_half(phi, h, 0)
        return var_line_solve(phi, 1 + 2 * h + 8 * W * M * dt * well_slope(phi), h, 0)
    raise ValueError(solver)


def cahn_hilliard_matrix_1d(c, M: float, eps: float, dt: float, dx: float) -> np.ndarray:
    """implicit_matrix_1d of CahnHilliard.py:20-71 with the coefficients of
    engine_CahnHilliardImplicit1D (:148-163): row j holds
    1 + a (2 s_j + 6 e2/dx^2) on the diagonal, -a (s_j + 4 e2/dx^2) at
    j -/+ 1 and a e2/dx^2 at j -/+ 2 (periodic), a = M dt / dx^2,
    s = 4c^2 - 6c + 2."""
    n = c.size
    if n < 5:
        raise ValueError("the periodic pentadiagonal solve needs >= 5 cells")
    idx2 = 1.0 / dx ** 2
    e2 = eps ** 2
    a = M * dt * idx2
    s = well_slope(c)
    m = np.zeros((n, n))
    j = np.arange(n)
    m[j, j] = 1 + a * (2 * s + 6 * e2 * idx2)
    nb = -a * (s + 4 * e2 * idx2)
    m[j, (j - 1) % n] = nb
    m[j, (j + 1) % n] = nb
    m[j, (j - 2) % n] = a * e2 * idx2
    m[j, (j + 2) % n] = a * e2 * idx2
    return m


def cahn_hilliard_implicit_step(c, solver: str, M: float, W: float, eps: float, dt: float,
                                dx: float, adi: bool, gmres: bool) -> np.ndarray:
    """One step of CahnHilliard.simulation_loop for the non-explicit solvers
    (CahnHilliard.py:382-421). 1-D implicit (:148-179) and Crank-Nicolson
    (:180-227: an explicit step of M times the Laplacian of mu, without dt as
    written, then the implicit solve with dt/2). The
    2-D / 3-D engines and IMEX call the three-argument matrix builder of the
    Allen-Cahn module, which CahnHilliard.py does not define (TypeError in the
    reference); their evident intent, the Allen-Cahn formulas they copy
    (:228-341), is what runs here."""
    c = np.asarray(c, dtype=np.float64)
    if c.ndim == 1 and solver in ("implicit", "crank-nicolson"):
        h = dt
        if solver == "crank-nicolson":
            h = dt / 2
            mu = -eps ** 2 * lap_periodic(c, dx) + (4 * c ** 3 - 6 * c ** 2 + 2 * c)
            c = c + M * (np.roll(mu, 1) + np.roll(mu, -1) - 2 * mu) / dx ** 2
        return np.linalg.solve(cahn_hilliard_matrix_1d(c, M, eps, h, dx), c)
    return allen_cahn_implicit_step(c, solver, M, W, eps, dt, dx, adi, gmres)


def lap_periodic(x, dx):
    out = np.zeros_like(x)
    for ax in range(x.ndim):
        out += np.roll(x, 1, ax) + np.roll(x, -1, ax) - 2 * x
    return out / dx ** 2


def run_phase(model: str, c0, steps: int, solver: str, M: float, W: float, eps: float,
              dt: float, dx: float, adi: bool, gmres: bool) -> np.ndarray:
    fn = allen_cahn_implicit_step if model == "allen_cahn" else cahn_hilliard_implicit_step
    c = np.asarray(c0, dtype=np.float64)
    for _ in range(steps):
        c = fn(c, solver, M, W, eps, dt, dx, adi, gmres)
    return c
