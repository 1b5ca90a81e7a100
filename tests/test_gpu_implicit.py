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
