"""Implicit and Crank-Nicolson diffusion on the GPU, through the C ABI and the
Diffusion engine, against the oracle (oracle/implicit_ref.py) and the
reference's own engine functions (tests/golden/implicit_*,
crank_nicolson_*).

Tolerances (relative L2 over the cells):
  * fp64 vs the FP64 oracle: <= 1e-12;
  * fp32 vs the FP64 oracle: <= 1e-5 (the precision target).
At sizes beyond the dense oracle: exact properties of the periodic systems
(every row of the operator sums to 1, so the field's sum is conserved; a
Fourier mode is an eigenvector with a known factor).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import implicit_ref as I
from tests.helpers import golden_names, load_golden, make_structs, rel_l2, to_dev, from_dev

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 1e-5
IMPLICIT = golden_names("implicit_") + golden_names("crank_nicolson_")


def _setup(shape, precision):
    import torch
    from pyphasefield_gb300 import _lib as L
    g, _, kshape, pitch = make_structs(shape, "PERIODIC")
    dtype = torch.float64 if precision == "fp64" else torch.float32
    nbytes = C.c_size_t()
    L.call("ppf_implicit_scratch_bytes", C.byref(g), 8 if precision == "fp64" else 4,
           C.byref(nbytes))
    scratch = torch.empty(max(16, nbytes.value), dtype=torch.uint8, device="cuda")
    return g, kshape, pitch, dtype, scratch


def run_implicit_gpu(c0, steps, solver, D, dt, dx, adi, precision="fp64", tol=0.0):
    import torch
    from pyphasefield_gb300 import _lib as L
    c0 = np.asarray(c0, dtype=np.float64)
    g, kshape, pitch, dtype, scratch = _setup(c0.shape, precision)
    a = to_dev(c0, kshape, pitch, dtype, "cuda")
    o, tmp = torch.zeros_like(a), torch.zeros_like(a)
    sfx = "f64" if precision == "fp64" else "f32"
    p = L.PpfImplicitDiffusionParams(dx, dt, D, tol,
                                     L.PPF_SOLVER_CRANK_NICOLSON if solver == "crank-nicolson"
                                     else L.PPF_SOLVER_IMPLICIT, 1 if adi else 0)
    it = C.c_int32()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(steps):
        L.call(f"ppf_diffusion_implicit_step_{sfx}", C.byref(p), C.byref(g),
               C.c_void_p(a.data_ptr()), C.c_void_p(o.data_ptr()), C.c_void_p(tmp.data_ptr()),
               C.c_void_p(scratch.data_ptr()), scratch.numel(), C.byref(it), s)
        a, o = o, a
    torch.cuda.synchronize()
    return from_dev(a, kshape, c0.shape), it.value


def test_fixture_count():
    assert len(IMPLICIT) == 11


@pytest.mark.parametrize("name", IMPLICIT)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_reference_fixtures(cuda, name, precision):
    d = load_golden(name)
    m = d["meta"]
    out, _ = run_implicit_gpu(d["c0"], m["steps"], m["solver"], m["D"], m["dt"], m["dx"],
                              m["adi"], precision)
    exact = I.run(d["c0"], m["steps"], m["solver"], m["D"], m["dt"], m["dx"], m["adi"])
    tol = F64_TOL if precision == "fp64" else F32_TOL
    assert rel_l2(out, exact) < tol
    # the fixture is the reference's own output (GMRES: within its 1e-5 residual)
    assert rel_l2(out, d["out"]) < (1e-4 if m["gmres"] else max(tol, 1e-12))


def _line(shape, axis, alpha, eaxis, ealpha, precision, seed=0):
    import torch
    from pyphasefield_gb300 import _lib as L
    rng = np.random.default_rng(seed)
    c0 = rng.random(shape)
    g, kshape, pitch, dtype, scratch = _setup(shape, precision)
    a = to_dev(c0, kshape, pitch, dtype, "cuda")
    o = torch.zeros_like(a)
    sfx = "f64" if precision == "fp64" else "f32"
    kax = axis + (len(kshape) - len(shape))
    kex = eaxis + (len(kshape) - len(shape)) if eaxis >= 0 else -1
    L.call(f"ppf_line_solve_{sfx}", C.byref(g), kax, alpha, kex, ealpha,
           C.c_void_p(a.data_ptr()), C.c_void_p(o.data_ptr()), C.c_void_p(scratch.data_ptr()),
           scratch.numel(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    rhs = I.explicit_half(c0, ealpha, eaxis) if eaxis >= 0 else c0
    return from_dev(o, kshape, shape), I.line_solve(rhs, alpha, axis)


@pytest.mark.parametrize("shape,axis", [((1000,), 0), ((3,), 0), ((257, 300), 1),
                                        ((300, 257), 0), ((33, 40), 0), ((40, 33), 1),
                                        ((9, 70, 37), 0), ((9, 70, 37), 1), ((9, 70, 37), 2),
                                        # 33, 35 and 18 segments per line: the carry pass
                                        # runs several 32-segment batches; 532 segments:
                                        # more than the register-resident carry holds
                                        ((1056, 40), 0), ((1093, 20), 0), ((3, 9000), 1),
                                        ((17000, 8), 0)])
@pytest.mark.parametrize("alpha", [0.05, 2.0, 500.0])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_line_solve_every_axis(cuda, shape, axis, alpha, precision):
    got, ref = _line(shape, axis, alpha, -1, 0.0, precision)
    assert rel_l2(got, ref) < (F64_TOL if precision == "fp64" else 2e-6)


@pytest.mark.parametrize("shape,axis,eaxis", [((64, 50), 0, 0), ((64, 50), 1, 1),
                                              ((64, 50), 0, 1), ((64, 50), 1, 0),
                                              ((12, 20, 36), 1, 0), ((12, 20, 36), 0, 1),
                                              ((12, 20, 36), 2, 2), ((12, 20, 36), 2, 0),
                                              ((12, 20, 36), 0, 2), ((700,), 0, 0)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_line_solve_with_explicit_half(cuda, shape, axis, eaxis, precision):
    got, ref = _line(shape, axis, 0.7, eaxis, 0.7, precision, seed=3)
    assert rel_l2(got, ref) < (F64_TOL if precision == "fp64" else 2e-6)


@pytest.mark.parametrize("shape", [(64, 48), (20, 24, 28)])
@pytest.mark.parametrize("alpha", [0.1, 5.0, 200.0])
@pytest.mark.parametrize("cn", [False, True])
def test_periodic_solve_matches_fft(cuda, shape, alpha, cn):
    import torch
    from pyphasefield_gb300 import _lib as L
    c0 = np.random.default_rng(5).random(shape)
    for precision in ("fp64", "fp32"):
        g, kshape, pitch, dtype, _ = _setup(shape, precision)
        a = to_dev(c0, kshape, pitch, dtype, "cuda")
        o, t = torch.zeros_like(a), torch.zeros_like(a)
        it = C.c_int32()
        sfx = "f64" if precision == "fp64" else "f32"
        L.call(f"ppf_periodic_solve_{sfx}", C.byref(g), alpha, alpha if cn else 0.0, 0.0 + (
            1e-14 if precision == "fp64" else 1e-7), C.c_void_p(a.data_ptr()),
            C.c_void_p(o.data_ptr()), C.c_void_p(t.data_ptr()), C.byref(it),
            C.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        rhs = I.explicit_full(c0, alpha) if cn else c0
        ref = I.full_solve_fft(rhs, alpha)
        assert it.value == I.chebyshev_plan(alpha, len(shape),
                                            1e-14 if precision == "fp64" else 1e-7)[0]
        assert rel_l2(from_dev(o, kshape, shape), ref) < (F64_TOL if precision == "fp64"
                                                           else F32_TOL), precision


def _mode(shape, ks):
    grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    theta = [2 * np.pi * k * gi / n for k, gi, n in zip(ks, grids, shape)]
    return np.cos(sum(theta)), [2 * np.pi * k / n for k, n in zip(ks, shape)]


@pytest.mark.parametrize("solver,adi", [("implicit", True), ("crank-nicolson", True),
                                        ("implicit", False), ("crank-nicolson", False)])
def test_fourier_mode_and_mass_at_scale(cuda, solver, adi):
    """4096 x 2048 (32 MiB in fp32): a Fourier mode decays by its known factor
    and the sum of a random field is conserved."""
    shape = (4096, 2048)
    D, dt, dx = 1.0, 3.0, 1.0
    a = (0.5 if solver == "crank-nicolson" else 1.0) * D * dt / dx ** 2
    c0, th = _mode(shape, (3, 5))
    lam = [2 * a * (1 - np.cos(t)) for t in th]
    if solver == "implicit":
        fac = np.prod([1 / (1 + l) for l in lam]) if adi else 1 / (1 + sum(lam))
    else:
        fac = (np.prod([(1 - l) / (1 + l) for l in lam]) if adi
               else (1 - sum(lam)) / (1 + sum(lam)))
    out, _ = run_implicit_gpu(c0, 1, solver, D, dt, dx, adi, "fp32")
    assert np.abs(out - fac * c0).max() < 2e-6
    rng = np.random.default_rng(1)
    r0 = rng.random(shape)
    out, _ = run_implicit_gpu(r0, 2, solver, D, dt, dx, adi, "fp32")
    assert abs(out.sum() - r0.sum()) / r0.sum() < 2e-6


def test_invalid_arguments_rejected(cuda):
    import torch
    from pyphasefield_gb300 import _lib as L
    g, kshape, pitch, dtype, scratch = _setup((16, 16), "fp32")
    a = torch.zeros(kshape[:-1] + (pitch,), device="cuda")
    o = torch.zeros_like(a)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    with pytest.raises(L.PpfError, match="scratch"):
        L.call("ppf_line_solve_f32", C.byref(g), 0, 1.0, -1, 0.0, vp(a), vp(o), vp(scratch), 4, s)
    with pytest.raises(L.PpfError, match="differ"):
        L.call("ppf_line_solve_f32", C.byref(g), 0, 1.0, 0, 1.0, vp(a), vp(a), vp(scratch),
               scratch.numel(), s)
    with pytest.raises(L.PpfError, match="distinct"):
        L.call("ppf_periodic_solve_f32", C.byref(g), 1.0, 0.0, 1e-7, vp(a), vp(o), None, None, s)
    g2, kshape2, pitch2, _, scratch2 = _setup((2, 16), "fp32")
    b = torch.zeros(kshape2[:-1] + (pitch2,), device="cuda")
    with pytest.raises(L.PpfError, match=">= 3"):
        L.call("ppf_line_solve_f32", C.byref(g2), 0, 1.0, -1, 0.0, vp(b), vp(b), vp(scratch2),
               scratch2.numel(), s)
    p = L.PpfImplicitDiffusionParams(1.0, 1.0, 1.0, 0.0, 7, 0)
    with pytest.raises(L.PpfError, match="solver"):
        L.call("ppf_diffusion_implicit_step_f32", C.byref(p), C.byref(g), vp(a), vp(o), None,
               vp(scratch), scratch.numel(), None, s)
    torch.cuda.synchronize()


@pytest.mark.parametrize("solver,adi,shape", [("implicit", True, (40, 36)),
                                              ("crank-nicolson", True, (12, 10, 14)),
                                              ("implicit", False, (30, 26)),
                                              ("crank-nicolson", False, (50,))])
def test_engine_solver_keys(cuda, solver, adi, shape):
    """DiffusionGB300 with user_data solver / adi / gmres, advanced in captured
    graphs, equals the oracle (the reference's Diffusion.simulation_loop
    dispatch, Engines/Diffusion.py:671-720)."""
    from pyphasefield_gb300.engines import DiffusionGB300
    rng = np.random.default_rng(9)
    c0 = rng.random(shape)
    sim = DiffusionGB300(dimensions=list(shape), dx=1.0, dt=2.0,
                         user_data={"D": 0.5, "solver": solver, "adi": adi, "gmres": True,
                                    "precision": "fp64", "graph_chunk": 4})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[sim.fields[0]._slice] = c0
    sim.simulate(10)
    sim.retrieve_fields_from_GPU()
    ref = I.run(c0, 10, solver, 0.5, 2.0, 1.0, adi)
    assert rel_l2(sim.fields[0].get_cells(), ref) < F64_TOL
    assert sim.time_step_counter == 10


# ---------------------------------------------------------------------------
# Allen-Cahn / Cahn-Hilliard implicit engines (CahnAllen.py:137-267,
# CahnHilliard.py:148-341)

PHASE = golden_names("phase_implicit_")
_PSOLVER = {"implicit": 1, "crank-nicolson": 2, "imex": 3}


def run_phase_gpu(model, c0, steps, solver, M, W, eps, dt, dx, adi, gmres, precision="fp64"):
    import torch
    from pyphasefield_gb300 import _lib as L
    c0 = np.asarray(c0, dtype=np.float64)
    g, _, kshape, pitch = make_structs(c0.shape, "PERIODIC")
    dtype = torch.float64 if precision == "fp64" else torch.float32
    nbytes = C.c_size_t()
    L.call("ppf_phase_implicit_scratch_bytes", C.byref(g), 8 if precision == "fp64" else 4,
           C.byref(nbytes))
    scratch = torch.empty(max(16, nbytes.value), dtype=torch.uint8, device="cuda")
    a = to_dev(c0, kshape, pitch, dtype, "cuda")
    o, tmp = torch.zeros_like(a), torch.zeros_like(a)
    p = L.PpfImplicitPhaseParams(dx, dt, M, W, eps, 0.0,
                                 L.PPF_MODEL_ALLEN_CAHN if model == "allen_cahn"
                                 else L.PPF_MODEL_CAHN_HILLIARD, _PSOLVER[solver],
                                 1 if adi else 0, 1 if gmres else 0, 0, 0)
    it = C.c_int32()
    sfx = "f64" if precision == "fp64" else "f32"
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(steps):
        L.call(f"ppf_phase_implicit_step_{sfx}", C.byref(p), C.byref(g),
               C.c_void_p(a.data_ptr()), C.c_void_p(o.data_ptr()), C.c_void_p(tmp.data_ptr()),
               C.c_void_p(scratch.data_ptr()), scratch.numel(), C.byref(it), s)
        a, o = o, a
    torch.cuda.synchronize()
    return from_dev(a, kshape, c0.shape)


def test_phase_fixture_count():
    assert len(PHASE) == 11


@pytest.mark.parametrize("name", PHASE)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_phase_reference_fixtures(cuda, name, precision):
    d = load_golden(name)
    m = d["meta"]
    p = m["params"]
    args = (m["model"], d["c0"], m["steps"], m["solver"], p["M"], p["W"], p["epsilon"], m["dt"],
            m["dx"], m["adi"], m["gmres"])
    out = run_phase_gpu(*args, precision=precision)
    exact = I.run_phase(*args)
    tol = F64_TOL if precision == "fp64" else F32_TOL
    assert rel_l2(out, exact) < tol
    assert rel_l2(out, d["out"]) < (1e-3 if m["gmres"] else max(tol, 1e-12))


def _var_line(shape, axis, alpha, shared, expl, precision, seed=0):
    import torch
    from pyphasefield_gb300 import _lib as L
    rng = np.random.default_rng(seed)
    c0 = rng.random(shape)
    g, kshape, pitch, dtype, _ = _setup(shape, precision)
    nbytes = C.c_size_t()
    L.call("ppf_phase_implicit_scratch_bytes", C.byref(g), 8 if precision == "fp64" else 4,
           C.byref(nbytes))
    scratch = torch.empty(max(16, nbytes.value), dtype=torch.uint8, device="cuda")
    a = to_dev(c0, kshape, pitch, dtype, "cuda")
    o = torch.zeros_like(a)
    n = shape[axis]
    dbase, dcoef = 1 + 2 * alpha, 0.3
    dv = None
    dvec = None
    if shared:
        dv = 1 + 2 * alpha + 0.5 * rng.random(n)
        dvec = torch.tensor(dv, dtype=dtype, device="cuda")
    sfx = "f64" if precision == "fp64" else "f32"
    kax = axis + (len(kshape) - len(shape))
    L.call(f"ppf_var_line_solve_{sfx}", C.byref(g), kax, alpha, dbase, dcoef,
           C.c_void_p(dvec.data_ptr()) if shared else None, 1 if expl else 0, 0.6 * alpha,
           C.c_void_p(a.data_ptr()), C.c_void_p(o.data_ptr()), C.c_void_p(scratch.data_ptr()),
           scratch.numel(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    rhs = I.explicit_half(c0, 0.6 * alpha, axis) if expl else c0
    diag = dv if shared else dbase + dcoef * I.well_slope(rhs)
    return from_dev(o, kshape, shape), I.var_line_solve(rhs, diag, alpha, axis)


@pytest.mark.parametrize("shape,axis", [((3,), 0), ((33,), 0), ((34,), 0), ((1000,), 0),
                                        ((65, 20), 0), ((20, 65), 1), ((64, 9), 0),
                                        ((7, 40, 97), 0), ((7, 40, 97), 1), ((7, 40, 97), 2)])
@pytest.mark.parametrize("alpha", [0.05, 3.0, 400.0])
@pytest.mark.parametrize("variant", ["cell", "shared", "expl"])
def test_var_line_solve(cuda, shape, axis, alpha, variant):
    for precision in ("fp64", "fp32"):
        got, ref = _var_line(shape, axis, alpha, variant == "shared", variant == "expl",
                             precision, seed=len(shape) + axis)
        # float: the system's condition number grows like alpha (its smallest
        # eigenvalue stays near 1, its largest is about 1 + 4 alpha)
        tol = F64_TOL if precision == "fp64" else 2e-6 * max(1.0, alpha / 20)
        assert rel_l2(got, ref) < tol, precision


@pytest.mark.parametrize("shape,dt,dx,seed", [((14, 12), 0.5, 3.0, 0), ((64, 80), 0.6, 2.5, 1),
                                              ((300, 257), 1.0, 3.0, 2)])
def test_full_allen_cahn_system_beyond_the_bound_minres(cuda, shape, dt, dx, seed):
    """16 W M dt >= 4: the full 2-D system may be indefinite (here half the
    cells sit at phi = 0.75, the double well's most negative slope, and the
    matrix has negative eigenvalues) and the Chebyshev bound fails; the
    library solves it with MINRES in one persistent launch. Against the
    exact dense solve (small grids) or the system's own residual."""
    import torch
    from pyphasefield_gb300 import _lib as L
    rng = np.random.default_rng(seed)
    c0 = np.where(rng.random(shape) > 0.5, 0.75, 0.2) + 0.01 * (rng.random(shape) - 0.5)
    M, W, eps = 0.7, 1.3, 1.1
    assert 16 * W * M * dt >= 4
    args = ("allen_cahn", c0, 1, "implicit", M, W, eps, dt, dx, False, True)
    a = M * dt * eps ** 2 / dx ** 2
    d = 1 + 4 * a + 16 * W * M * dt * (4 * c0 * c0 - 6 * c0 + 2)

    def residual(x):
        ax = d * x - a * (np.roll(x, 1, 0) + np.roll(x, -1, 0) + np.roll(x, 1, 1)
                          + np.roll(x, -1, 1))
        return np.linalg.norm(ax - c0) / np.linalg.norm(c0)

    for precision, tol in (("fp64", F64_TOL), ("fp32", F32_TOL)):
        v = C.c_int32()
        L.call("ppf_status_take", C.byref(v))
        out = run_phase_gpu(*args, precision=precision)
        L.call("ppf_status_take", C.byref(v))
        assert v.value == 0, v.value  # converged: no status bit
        assert residual(out) < (1e-12 if precision == "fp64" else 1e-5)
        if c0.size <= 5000:
            assert rel_l2(out, I.run_phase(*args)) < tol
    assert (out < 0).any()  # the indefinite step overshoots below phi = 0


def test_minres_reports_an_unconverged_solve(cuda):
    """An iteration cap too small for the system (3 iterations): the solve
    sets PPF_STATUS_NOT_CONVERGED instead of passing off its iterate as
    converged."""
    import torch
    from pyphasefield_gb300 import _lib as L
    rng = np.random.default_rng(3)
    c0 = np.where(rng.random((64, 64)) > 0.5, 0.75, 0.2)
    g, _, kshape, pitch = make_structs(c0.shape, "PERIODIC")
    nbytes = C.c_size_t()
    L.call("ppf_phase_implicit_scratch_bytes", C.byref(g), 8, C.byref(nbytes))
    scratch = torch.empty(nbytes.value, dtype=torch.uint8, device="cuda")
    a = to_dev(c0, kshape, pitch, torch.float64, "cuda")
    o, tmp = torch.zeros_like(a), torch.zeros_like(a)
    p = L.PpfImplicitPhaseParams(2.5, 0.6, 0.7, 1.3, 1.1, 0.0, L.PPF_MODEL_ALLEN_CAHN, 1, 0, 1,
                                 3, 0)
    v = C.c_int32()
    L.call("ppf_status_take", C.byref(v))
    it = C.c_int32()
    L.call("ppf_phase_implicit_step_f64", C.byref(p), C.byref(g), C.c_void_p(a.data_ptr()),
           C.c_void_p(o.data_ptr()), C.c_void_p(tmp.data_ptr()), C.c_void_p(scratch.data_ptr()),
           scratch.numel(), C.byref(it), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    L.call("ppf_status_take", C.byref(v))
    assert v.value & L.PPF_STATUS_NOT_CONVERGED


def test_cahn_hilliard_1d_pentadiagonal_large(cuda):
    rng = np.random.default_rng(12)
    c0 = 0.5 + 0.3 * (rng.random(2000) - 0.5)
    args = ("cahn_hilliard", c0, 2, "implicit", 1.0, 1.0, 1.0, 0.5, 1.0, False, False)
    exact = I.run_phase(*args)
    assert rel_l2(run_phase_gpu(*args, precision="fp64"), exact) < F64_TOL
    assert rel_l2(run_phase_gpu(*args, precision="fp32"), exact) < F32_TOL


@pytest.mark.parametrize("cls,solver,adi,gmres,shape", [
    ("CahnAllenGB300", "implicit", True, False, (40, 36)),
    ("CahnAllenGB300", "implicit", False, True, (24, 20)),
    ("CahnAllenGB300", "crank-nicolson", True, False, (30, 34)),
    ("CahnAllenGB300", "implicit", True, False, (10, 12, 14)),
    ("CahnAllenGB300", "imex", False, False, (90,)),
    ("CahnHilliardGB300", "crank-nicolson", False, False, (80,))])
def test_phase_engine_solver_keys(cuda, cls, solver, adi, gmres, shape):
    """The Allen-Cahn / Cahn-Hilliard engines with solver / adi / gmres keys,
    through captured graphs, equal the oracle."""
    import pyphasefield_gb300 as P
    rng = np.random.default_rng(4)
    c0 = 0.5 + 0.4 * (rng.random(shape) - 0.5)
    ud = {"M": 0.7, "W": 1.3, "epsilon": 1.1, "solver": solver, "adi": adi, "gmres": gmres,
          "precision": "fp64", "graph_chunk": 4}
    # the full 2-D solve needs 16 W M dt < 4; the IMEX engine's -2 phi term
    # (as the reference writes it) makes larger steps run away
    dt = 0.005 if solver == "imex" else (0.1 if gmres and not adi else 0.3)
    sim = getattr(P, cls)(dimensions=list(shape), dx=1.2, dt=dt, user_data=ud)
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[sim.fields[0]._slice] = c0
    sim.simulate(9)
    sim.retrieve_fields_from_GPU()
    model = "allen_cahn" if cls == "CahnAllenGB300" else "cahn_hilliard"
    ref = I.run_phase(model, c0, 9, solver, 0.7, 1.3, 1.1, dt, 1.2, adi, gmres)
    assert np.isfinite(ref).all()
    # nine steps of a stiff nonlinear map (16 W M dt = 4.4) amplify the
    # rounding-order differences of each solve (1e-15) to about 1e-10
    assert rel_l2(sim.fields[0].get_cells(), ref) < 1e-9
