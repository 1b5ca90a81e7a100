"""The engines through the reference-facing API (Simulation subclasses):
lifecycle hooks, CUDA-graph stepping, autosave/load, precision, diagnostics.
Tolerances as in test_gpu_kernels: fp32 within 1e-5 relative L2 of the FP64
oracle, fp64 within 1e-12; graph vs eager stepping bit for bit."""
import numpy as np
import pytest

from oracle import restate
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def _warren(shape, phi0, c0, bc="NEUMANN", **ud):
    from pyphasefield_gb300 import Warren1995GB300
    sim = Warren1995GB300(dimensions=list(shape), dx=4.6e-8, boundary_conditions=bc,
                          user_data=dict(ud))
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = phi0
    sim.fields[1].data[1:-1, 1:-1] = c0
    return sim


def _seeded(shape, seed=0):
    rng = np.random.default_rng(seed)
    phi0 = np.ones(shape)
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    phi0[(yy - shape[0] / 2 + 0.5) ** 2 + (xx - shape[1] / 2 + 0.5) ** 2 < 36] = 0.0
    c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    return phi0, c0


def test_warren_engine_matches_oracle_graph_and_eager(cuda):
    shape = (64, 72)
    phi0, c0 = _seeded(shape)
    params = dict(restate.WARREN_DEFAULTS, alpha=0.3)
    ref = restate.run_warren(phi0, c0, 50, "NEUMANN", 4.6e-8, params, seed=7)
    a = _warren(shape, phi0, c0, seed=7, graph_chunk=8)
    a.simulate(50)
    a.retrieve_fields_from_GPU()
    b = _warren(shape, phi0, c0, seed=7, use_graph=False)
    for _ in range(5):
        b.simulate(10)
    b.retrieve_fields_from_GPU()
    for f in (0, 1):
        np.testing.assert_array_equal(a.fields[f].get_cells(), b.fields[f].get_cells())
    assert rel_l2(a.fields[0].get_cells(), ref[0]) < 1e-5
    assert rel_l2(a.fields[1].get_cells(), ref[1]) < 1e-5
    assert a.time_step_counter == 50 and b.time_step_counter == 50
    # ghosts refreshed on the host with the no-flux rule
    d = a.fields[0].data
    np.testing.assert_array_equal(d[0, 1:-1], d[1, 1:-1])
    np.testing.assert_array_equal(d[1:-1, -1], d[1:-1, -2])


def test_warren_engine_fp64_tight(cuda):
    shape = (40, 50)
    phi0, c0 = _seeded(shape, 1)
    params = dict(restate.WARREN_DEFAULTS, alpha=0.3)
    ref = restate.run_warren(phi0, c0, 30, ["PERIODIC", "NEUMANN"], 4.6e-8, params, seed=2)
    sim = _warren(shape, phi0, c0, bc=["PERIODIC", "NEUMANN"], seed=2, precision="fp64",
                  graph_chunk=4)
    sim.simulate(30)
    sim.retrieve_fields_from_GPU()
    assert rel_l2(sim.fields[0].get_cells(), ref[0]) < 1e-12
    assert rel_l2(sim.fields[1].get_cells(), ref[1]) < 1e-12


def test_autosave_and_load_round_trip(cuda, tmp_path):
    from pyphasefield_gb300 import DiffusionGB300
    rng = np.random.default_rng(3)
    c0 = rng.random((30, 40))
    sim = DiffusionGB300(dimensions=[30, 40], dx=1.0, dt=0.1, boundary_conditions="PERIODIC",
                         save_path=str(tmp_path), autosave=True, autosave_rate=7,
                         user_data={"D": 1.0, "graph_chunk": 4})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = c0
    sim.simulate(20)
    assert sorted(p.name for p in tmp_path.glob("*.npz")) == ["step_14.npz", "step_7.npz"]
    ref14 = restate.run_single("diffusion", c0, 14, "PERIODIC", 1.0, 0.1, D=1.0)
    ref7 = restate.run_single("diffusion", c0, 7, "PERIODIC", 1.0, 0.1, D=1.0)
    with np.load(tmp_path / "step_14.npz") as z:
        assert rel_l2(z["c"], ref14) < 1e-5
    with np.load(tmp_path / "step_7.npz") as z:
        assert rel_l2(z["c"], ref7) < 1e-5
    # the checkpoints are written while stepping on; simulate() returns with
    # Field.data at the last autosaved step, as the reference's engines do
    assert rel_l2(sim.fields[0].get_cells(), ref14) < 1e-5
    again = DiffusionGB300(dimensions=[30, 40], dx=1.0, dt=0.1, boundary_conditions="PERIODIC",
                           user_data={"D": 1.0})
    again.load_simulation(file_path=str(tmp_path / "step_14.npz"))
    assert again.time_step_counter == 14
    again.simulate(6)
    again.retrieve_fields_from_GPU()
    sim.retrieve_fields_from_GPU()
    np.testing.assert_array_equal(again.fields[0].get_cells(), sim.fields[0].get_cells())


@pytest.mark.parametrize("depth", [1, 4])
def test_diffusion_engine_temporal_depth(cuda, depth):
    from pyphasefield_gb300 import DiffusionGB300
    rng = np.random.default_rng(0)
    c0 = 0.5 + 0.01 * rng.standard_normal((256, 256))
    sim = DiffusionGB300(dimensions=[256, 256], dx=1.0, dt=0.2, boundary_conditions="PERIODIC",
                         user_data={"D": 1.0, "temporal_depth": depth, "graph_chunk": 16})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = c0
    sim.simulate(1000)
    sim.retrieve_fields_from_GPU()
    ref = restate.run_single("diffusion", c0, 1000, "PERIODIC", 1.0, 0.2, D=1.0)
    assert rel_l2(sim.fields[0].get_cells(), ref) < 1e-5


def test_cahn_hilliard_engine_exact_mass_and_parity(cuda):
    from pyphasefield_gb300 import CahnHilliardGB300
    rng = np.random.default_rng(0)
    shape = (40, 36, 44)
    c0 = 0.5 + rng.uniform(-0.05, 0.05, shape)
    sim = CahnHilliardGB300(dimensions=list(shape), dx=1.0, dt=0.01,
                            boundary_conditions="PERIODIC",
                            user_data={"M": 1.0, "epsilon": 1.0, "graph_chunk": 16})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1, 1:-1] = c0
    sim.simulate(300)
    mass = sim.collect_mass_history()
    assert len(mass) == 300
    q = 2.0 ** -24
    m0 = (np.rint((c0 - 0.5) / q) * q + 0.5).sum()
    assert np.all(mass == mass[0]) and abs(mass[0] - m0) <= 1e-9 * m0
    sim.retrieve_fields_from_GPU()
    c0q = np.rint((c0 - 0.5) / q) * q + 0.5
    ref = restate.run_single("cahn_hilliard", c0q, 300, "PERIODIC", 1.0, 0.01, M=1.0, epsilon=1.0)
    assert rel_l2(sim.fields[0].get_cells(), ref) < 1e-5
    assert sim.status_flags() == 0


def test_allen_cahn_engine_3d_and_fp64(cuda):
    from pyphasefield_gb300 import AllenCahnGB300
    rng = np.random.default_rng(4)
    c0 = rng.random((20, 24, 28))
    for prec, tol in (("fp32", 1e-5), ("fp64", 1e-12)):
        sim = AllenCahnGB300(dimensions=[20, 24, 28], dx=1.0, dt=0.05,
                             boundary_conditions=["NEUMANN", "PERIODIC", "DIRCHLET"],
                             user_data={"precision": prec, "graph_chunk": 4})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1, 1:-1] = c0
        sim.simulate(25)
        sim.retrieve_fields_from_GPU()
        ref = restate.run_single("allen_cahn", c0, 25, ["NEUMANN", "PERIODIC", "DIRCHLET"], 1.0,
                                 0.05, M=0.1, epsilon=1.0, W=1.0)
        assert rel_l2(sim.fields[0].get_cells(), ref) < tol


def test_engine_rejections(cuda):
    from pyphasefield_gb300 import CahnHilliardGB300, DiffusionGB300
    ch = CahnHilliardGB300(dimensions=[16, 16], dx=1.0, dt=0.01, boundary_conditions="DIRCHLET")
    ch.initialize_fields_and_imported_data()
    with pytest.raises(RuntimeError, match="PERIODIC and NEUMANN"):
        ch.simulate(1)
    d = DiffusionGB300(dimensions=[16, 16], dx=1.0, dt=0.1, boundary_conditions="NEUMANN",
                       user_data={"solver": "multigrid"})
    d.initialize_fields_and_imported_data()
    with pytest.raises(ValueError, match="solver must be one of"):
        d.simulate(1)
    d2 = DiffusionGB300(dimensions=[16, 16], dx=1.0, dt=0.1, boundary_conditions="NEUMANN")
    d2.initialize_fields_and_imported_data()
    d2._boundary_conditions_array[0][0, 3] = 0.5  # non-uniform face
    with pytest.raises(NotImplementedError, match="non-uniform"):
        d2.simulate(1)


def test_linear_gradient_temperature_bookkeeping(cuda):
    """LINEAR_GRADIENT (simulation.py:134-155, 313-315): the temperature
    field starts as initial_T + gradients and advances dTdt * dt per step;
    the engines do not read it (Warren1995 takes the scalar T), so the fields
    equal an isothermal run bit for bit."""
    from pyphasefield_gb300 import DiffusionGB300
    rng = np.random.default_rng(3)
    c0 = rng.random((40, 56))
    runs = []
    for ttype in ("ISOTHERMAL", "LINEAR_GRADIENT"):
        d = DiffusionGB300(dimensions=[40, 56], dx=0.5, dt=0.05, boundary_conditions="PERIODIC",
                           temperature_type=ttype, initial_T=1000.0, dTdx=2.0, dTdy=-1.0,
                           dTdt=-3.0, user_data={"D": 1.0, "graph_chunk": 8})
        d.initialize_fields_and_imported_data()
        d.fields[0].data[1:-1, 1:-1] = c0
        t_init = d.temperature.get_cells().copy()
        d.simulate(37)
        d.retrieve_fields_from_GPU()
        runs.append((d.fields[0].get_cells().copy(), t_init, d.temperature.get_cells().copy()))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    (_, t0, t1) = runs[1]
    np.testing.assert_allclose(t1, t0 + 37 * -3.0 * 0.05, rtol=0, atol=1e-9)
    assert t0[0, 1] - t0[0, 0] == pytest.approx(2.0 * 0.5)  # dTdx along the last axis
    np.testing.assert_array_equal(runs[0][2], runs[0][1])  # isothermal stays put


def test_xdmf_temperature_is_rejected(cuda):
    from pyphasefield_gb300 import DiffusionGB300
    d = DiffusionGB300(dimensions=[16, 16], dx=1.0, dt=0.1, boundary_conditions="PERIODIC",
                       user_data={"D": 1.0})
    d.initialize_fields_and_imported_data()
    d._temperature_type = "XDMF_FILE"
    with pytest.raises(NotImplementedError, match="meshio"):
        d.simulate(1)


def test_async_autosave_many_checkpoints(cuda, tmp_path):
    """Checkpoints every 3 steps (snapshot slots reused while earlier writes
    may still run): every file holds its own step."""
    from pyphasefield_gb300 import CahnAllenGB300
    rng = np.random.default_rng(4)
    c0 = rng.random((48, 33))
    sim = CahnAllenGB300(dimensions=[48, 33], dx=1.0, dt=0.1, boundary_conditions="NEUMANN",
                         save_path=str(tmp_path), autosave=True, autosave_rate=3,
                         user_data={"graph_chunk": 2})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = c0
    sim.simulate(16)
    names = sorted(int(p.stem.split("_")[1]) for p in tmp_path.glob("step_*.npz"))
    assert names == [3, 6, 9, 12, 15]
    for n in names:
        ref = restate.run_single("allen_cahn", c0, n, "NEUMANN", 1.0, 0.1, M=0.1, epsilon=1.0,
                                 W=1.0)
        with np.load(tmp_path / f"step_{n}.npz") as z:
            assert rel_l2(z["phi"], ref) < 1e-5, n
