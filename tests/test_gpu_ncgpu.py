"""NCGPU on the GPU (csrc/ncgpu.cu) through the C ABI and the engine, against
the fixtures made by the reference's own kernels (tests/golden/ncgpu_*) and
the oracle (oracle/ncgpu_ref.py).

Tolerances (relative L2 per field): fp64 <= 1e-8 (the reference's
forward-difference dG/dc amplifies rounding-order differences of c by ~1e6,
see tests/test_ncgpu_oracle.py); fp32 <= 1e-5."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import ncgpu_ref as N
from tests.helpers import from_dev, make_structs, rel_l2, to_dev

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
TDB = GOLDEN / "ncgpu_nicu.tdb"
TOL = {"fp64": 1e-8, "fp32": 1e-5}


def params_struct(dx, noise_scale=1.0, tdb=TDB, variant=0):
    from pyphasefield_gb300.engines.ncgpu import ncgpu_parameters, params_struct as ps
    from pyphasefield_gb300.tdb import Database
    db = Database(tdb)
    ud = ncgpu_parameters(db, dx)
    if variant:
        ud.update(eqbar=0.1 * ud["ebar"], noise_phi=1.0, noise_q=1.0)
    return ps(db, ud, dx, noise_scale, variant)


def run_gpu(fields, T, steps, dx, seed, bc, precision, noise_scale=1.0, tdb=TDB, tables=True,
            variant=0, dT_step=0.0):
    """`steps` steps through ppf_ncgpu_step_*; tables: the pure-element
    energies from ppf_ncgpu_tables_* (False: evaluated in every step);
    dT_step: the temperature rises by it after every step
    (ppf_ncgpu_temperature_advance_*)."""
    import torch
    from pyphasefield_gb300 import _lib as L
    shape = fields[0].shape
    g, b, kshape, pitch = make_structs(shape, bc)
    dtype = torch.float64 if precision == "fp64" else torch.float32
    a = [to_dev(f, kshape, pitch, dtype, "cuda") for f in fields]
    o = [torch.zeros_like(t) for t in a]
    temp = to_dev(T, kshape, pitch, dtype, "cuda")
    transfer = torch.zeros((2 * len(fields) - 5,) + tuple(a[0].shape), dtype=dtype, device="cuda")
    p = params_struct(dx, noise_scale, tdb, variant)
    sfx = "f64" if precision == "fp64" else "f32"
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    tab = None
    if tables:
        tab = torch.empty((2 * p.ncomp + p.nexcess,) + tuple(a[0].shape), dtype=torch.float64,
                          device="cuda")
        L.call(f"ppf_ncgpu_tables_{sfx}", C.byref(p), C.byref(g), C.c_void_p(temp.data_ptr()),
               C.c_void_p(tab.data_ptr()), s)
    for k in range(steps):
        fin = (C.c_void_p * len(a))(*[t.data_ptr() for t in a])
        fout = (C.c_void_p * len(o))(*[t.data_ptr() for t in o])
        L.call(f"ppf_ncgpu_step_{sfx}", C.byref(p), C.byref(g), C.byref(b), fin, fout,
               C.c_void_p(temp.data_ptr()), C.c_void_p(None if tab is None else tab.data_ptr()),
               C.c_void_p(transfer.data_ptr()), C.c_uint64(seed), C.c_uint64(k), None, s)
        if dT_step:
            L.call(f"ppf_ncgpu_temperature_advance_{sfx}", C.byref(g),
                   C.c_void_p(temp.data_ptr()), C.c_double(dT_step), s)
        a, o = o, a
    torch.cuda.synchronize()
    return [from_dev(t, kshape, shape) for t in a]


@pytest.mark.parametrize("name", ["ncgpu_periodic", "ncgpu_neumann", "ncgpu_ninb"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("tables", [True, False])
def test_reference_fixtures(cuda, name, precision, tables):
    """Ni-Cu (ideal) and Ni-Nb (binary Redlich-Kister terms of orders 0-2)
    against the reference's kernels."""
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    T = np.full(z["phi0"].shape, m["T"])
    out = run_gpu([z["phi0"], z["q10"], z["q40"], z["c0"]], T, m["steps"], m["dx"], m["seed"],
                  m["bc"], precision, tables=tables, tdb=GOLDEN / m["tdb"])
    for got, key in zip(out, ("phi", "q1", "q4", "c")):
        assert rel_l2(got, z[key]) < TOL[precision], (key, rel_l2(got, z[key]))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_cooling_reference_fixture(cuda, precision):
    """A LINEAR_GRADIENT temperature that falls 5 K per step (dT/dt), against
    the reference's kernels with the temperature raised after every step as
    its update_thermal_gradient kernel does."""
    z = np.load(GOLDEN / "ncgpu_cooling.npz")
    m = json.loads(str(z["meta"]))
    out = run_gpu([z["phi0"], z["q10"], z["q40"], z["c0"]], z["T0"], m["steps"], m["dx"],
                  m["seed"], m["bc"], precision, tables=False, dT_step=m["dT_step"])
    for got, key in zip(out, ("phi", "q1", "q4", "c")):
        assert rel_l2(got, z[key]) < TOL[precision], (key, rel_l2(got, z[key]))


def test_cooling_engine_against_oracle(cuda):
    """NCGPUGB300 with temperature_type LINEAR_GRADIENT, dTdx and dTdt,
    through captured graphs (two chunks of two steps): against the oracle
    with the same per-step rise, and the host temperature field advanced by
    the same amount. (Over more steps fp64 parts at the 1e-7 level, as in
    test_gradient_run_against_oracle: the forward-difference dG/dc.)"""
    from pyphasefield_gb300 import NCGPUGB300
    shape, steps = (30, 28), 4
    tdb = N.Tdb(TDB)
    p = N.tdb_params(tdb, 4.6e-6)
    dTdt = -2.0 / p["dt"]  # -2 K per step
    sim = NCGPUGB300(dimensions=list(shape), dx=4.6e-6, tdb_path=str(TDB),
                     temperature_type="LINEAR_GRADIENT", initial_T=1578.0, dTdx=3000.0,
                     dTdt=dTdt, boundary_conditions="NEUMANN",
                     user_data={"seed": 4, "sim_type": "seed", "graph_chunk": 2,
                                "initial_concentration_array": [0.40831]})
    sim.initialize_fields_and_imported_data()
    T0 = sim.temperature.get_cells().copy()
    init = [f.get_cells().copy() for f in sim.fields]
    sim.simulate(steps)
    sim.retrieve_fields_from_GPU()
    ref = N.run(init, T0, steps, p, tdb, seed=4, bc="NEUMANN", dT_step=dTdt * sim.dt)
    for f, r, key in zip(sim.fields, ref, ("phi", "q1", "q4", "c")):
        assert rel_l2(f.get_cells(), r) < 1e-8, (key, rel_l2(f.get_cells(), r))
    np.testing.assert_allclose(sim.temperature.get_cells(), T0 + steps * dTdt * sim.dt,
                               rtol=1e-12)


@pytest.fixture(scope="module")
def gradient_case():
    """20 steps on 40 x 36 with a temperature gradient along x and a seed at
    30 degrees in a melt at 0.1 rad (oracle computed once)."""
    shape = (40, 36)
    tdb = N.Tdb(TDB)
    p = N.tdb_params(tdb, 4.6e-6)
    phi, q1, q4, c = N.seed_fields(shape, melt_angle=0.1, seed_angle=np.pi / 6, c0=0.40831)
    c = c + np.random.default_rng(3).uniform(-1e-3, 1e-3, shape)
    T = 1570.0 + 2.0 * np.arange(shape[1])[None, :] * np.ones(shape)
    ref4 = N.run([phi, q1, q4, c], T, 4, p, tdb, seed=5, bc="NEUMANN")
    ref20 = N.run(ref4, T, 16, p, tdb, seed=5, bc="NEUMANN", step0=4)
    return [phi, q1, q4, c], T, {4: ref4, 20: ref20}


@pytest.mark.parametrize("precision,steps,tol", [("fp64", 20, 1e-3), ("fp64", 4, 1e-8),
                                                 ("fp32", 4, 1e-5)])
def test_gradient_run_against_oracle(cuda, gradient_case, precision, steps, tol):
    """Every term of the kernel, the temperature-gradient terms included,
    against the oracle. Over 20 steps fp64 agrees to ~1e-4: the reference's
    forward-difference dG/dc (step 1e-7) turns one-ulp differences of the
    Gibbs energies (the device's log and fused multiply-adds against
    numpy's) into 1e-9 of dF/dc every step, and the kernel's thresholds
    (clamps of |grad q| and phi) turn those into jumps at single cells
    (the orientation fields part by up to 1e-2 over 20 steps). In fp32 the thresholds of
    the kernel (|grad q| clamped at beta, phi clamped to [1e-6, 1 - 1e-6])
    flip for some cells after ~6 steps, and the orientation fields part at
    the percent level: fp64 is the accurate path for this engine."""
    fields, T, ref = gradient_case
    out = run_gpu(fields, T, steps, 4.6e-6, 5, "NEUMANN", precision)
    for got, r, key in zip(out, ref[steps], ("phi", "q1", "q4", "c")):
        # after 20 steps the orientation fields carry the jumps of the
        # |grad q| clamp (cells whose |grad q| sits at beta = 1.5 / cm)
        t = 20 * tol if steps == 20 and key in ("q1", "q4") else tol
        assert rel_l2(got, r) < t, (key, rel_l2(got, r))


def test_tables_equal_the_per_step_evaluation(cuda, gradient_case):
    """The pure-element energies read from ppf_ncgpu_tables_f64 (a
    temperature that varies along x) give the same run as evaluating them
    in every step."""
    fields, T, _ = gradient_case
    a = run_gpu(fields, T, 4, 4.6e-6, 5, "NEUMANN", "fp64", tables=True)
    b = run_gpu(fields, T, 4, 4.6e-6, 5, "NEUMANN", "fp64", tables=False)
    for x, y in zip(a, b):
        assert rel_l2(x, y) < 1e-12


MULTI = ["ncgpu_ternary", "ncgpu_quaternary", "ncgpu_senary"]


@pytest.mark.parametrize("name", MULTI)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_multicomponent_reference_fixture(cuda, name, precision):
    """Three (Ni-Cu-Al), four and six components (Ni-Cu-Al plus pseudo
    elements): two, three and five concentration fields."""
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    nc = sum(1 for k in z.files if k.startswith("c0_"))
    T = np.full(z["phi0"].shape, m["T"])
    f = [z["phi0"], z["q10"], z["q40"]] + [z[f"c0_{j}"] for j in range(nc)]
    out = run_gpu(f, T, m["steps"], m["dx"], m["seed"], m["bc"], precision, tdb=GOLDEN / m["tdb"])
    keys = ["phi", "q1", "q4"] + [f"c_{j}" for j in range(nc)]
    for got, key in zip(out, keys):
        assert rel_l2(got, z[key]) < TOL[precision], (key, rel_l2(got, z[key]))


def test_noise_off_is_deterministic_and_noise_on_is_not(cuda):
    z = np.load(GOLDEN / "ncgpu_periodic.npz")
    T = np.full(z["phi0"].shape, 1574.0)
    f = [z["phi0"], z["q10"], z["q40"], z["c0"]]
    a = run_gpu(f, T, 3, 4.6e-6, 1, "PERIODIC", "fp64", noise_scale=0.0)
    b = run_gpu(f, T, 3, 4.6e-6, 2, "PERIODIC", "fp64", noise_scale=0.0)
    np.testing.assert_array_equal(a[3], b[3])
    c = run_gpu(f, T, 3, 4.6e-6, 2, "PERIODIC", "fp64", noise_scale=1.0)
    assert rel_l2(c[3], a[3]) > 1e-6


def test_engine_matches_oracle(cuda):
    """NCGPUGB300 (tdb_path, ISOTHERMAL 1574 K, sim_type seed) through
    captured graphs equals the oracle from the engine's own initial fields."""
    from pyphasefield_gb300 import NCGPUGB300
    shape = (24, 20)
    sim = NCGPUGB300(dimensions=list(shape), dx=4.6e-6, tdb_path=str(TDB),
                     temperature_type="ISOTHERMAL", initial_T=1574.0,
                     boundary_conditions="PERIODIC",
                     user_data={"sim_type": "seed", "initial_concentration_array": [0.40831],
                                "seed": 7, "precision": "fp64", "graph_chunk": 2})
    sim.initialize_fields_and_imported_data()
    init = [f.get_cells().copy() for f in sim.fields]
    sim.simulate(5)
    sim.retrieve_fields_from_GPU()
    tdb = N.Tdb(TDB)
    ref = N.run(init, np.full(shape, 1574.0), 5, N.tdb_params(tdb, 4.6e-6), tdb, seed=7,
                bc="PERIODIC")
    for f, r in zip(sim.fields, ref):
        assert rel_l2(f.get_cells(), r) < TOL["fp64"], f.name
    assert sim.time_step_counter == 5
    assert [f.name for f in sim.fields] == ["phi", "q1", "q4", "c_CU"]


def test_engine_six_components_matches_oracle(cuda):
    """The engine on the six-component database (five concentration fields,
    the initial_concentration_array of the reference) against the oracle."""
    from pyphasefield_gb300 import NCGPUGB300
    path = GOLDEN / "ncgpu_6comp.tdb"
    shape = (20, 18)
    sim = NCGPUGB300(dimensions=list(shape), dx=4.6e-6, tdb_path=str(path),
                     temperature_type="ISOTHERMAL", initial_T=1574.0,
                     boundary_conditions="NEUMANN",
                     user_data={"sim_type": "seed",
                                "initial_concentration_array": [0.05, 0.2, 0.3, 0.1, 0.15],
                                "seed": 4, "precision": "fp64", "graph_chunk": 2})
    sim.initialize_fields_and_imported_data()
    assert [f.name for f in sim.fields] == ["phi", "q1", "q4", "c_AL", "c_CU", "c_NI", "c_XA",
                                            "c_XB"]
    init = [f.get_cells().copy() for f in sim.fields]
    sim.simulate(4)
    sim.retrieve_fields_from_GPU()
    tdb = N.Tdb(path)
    ref = N.run(init, np.full(shape, 1574.0), 4, N.tdb_params(tdb, 4.6e-6), tdb, seed=4,
                bc="NEUMANN")
    for f, r in zip(sim.fields, ref):
        assert rel_l2(f.get_cells(), r) < TOL["fp64"], f.name


@pytest.mark.parametrize("name", ["ncgpu_new_periodic", "ncgpu_new_ternary"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ncgpu_new_reference_fixtures(cuda, name, precision):
    """PPF_NCGPU_VARIANT_NEW against Engines/NCGPU_new.py's own kernels:
    per-component dG/dc and noise, phase and orientation noise. In float32
    the binary periodic case parts by 1.3e-4 (relative L2) in q4: at step 2
    one interface cell's |grad q| falls on the other side of the beta clamp
    than in float64 and the jump spreads to ~30 cells (a float32 emulation
    of the kernel on the CPU gives 1.28e-4, the GPU 1.31e-4); that case is
    held to 1e-3, the others to the float tolerance."""
    tol = 1e-3 if (precision, name) == ("fp32", "ncgpu_new_periodic") else TOL[precision]
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    nc = sum(1 for k in z.files if k.startswith("c0_"))
    T = np.full(z["phi0"].shape, m["T"])
    f = [z["phi0"], z["q10"], z["q40"]] + [z[f"c0_{j}"] for j in range(nc)]
    out = run_gpu(f, T, m["steps"], m["dx"], m["seed"], m["bc"], precision, tdb=GOLDEN / m["tdb"],
                  variant=1)
    keys = ["phi", "q1", "q4"] + [f"c_{j}" for j in range(nc)]
    for got, key in zip(out, keys):
        assert rel_l2(got, z[key]) < tol, (key, rel_l2(got, z[key]))


def test_ncgpu_new_engine_matches_oracle(cuda):
    """NCGPU_newGB300 (sim_type seeds, melt angle) through captured graphs
    against the oracle's NCGPU_new variant."""
    from pyphasefield_gb300 import NCGPU_newGB300
    path = GOLDEN / "ncgpu_nicual.tdb"
    shape = (22, 24)
    sim = NCGPU_newGB300(dimensions=list(shape), dx=4.6e-6, tdb_path=str(path),
                         temperature_type="ISOTHERMAL", initial_T=1574.0,
                         boundary_conditions="NEUMANN",
                         user_data={"sim_type": "seeds", "number_of_seeds": 2, "melt_angle": 0.2,
                                    "initial_concentration_array": [0.05, 0.4], "seed": 6,
                                    "precision": "fp64", "graph_chunk": 2})
    sim.initialize_fields_and_imported_data()
    init = [f.get_cells().copy() for f in sim.fields]
    sim.simulate(4)
    sim.retrieve_fields_from_GPU()
    tdb = N.Tdb(path)
    ref = N.run(init, np.full(shape, 1574.0), 4, N.tdb_params(tdb, 4.6e-6, variant="NCGPU_new"),
                tdb, seed=6, bc="NEUMANN", variant="NCGPU_new")
    for f, r in zip(sim.fields, ref):
        assert rel_l2(f.get_cells(), r) < TOL["fp64"], f.name
