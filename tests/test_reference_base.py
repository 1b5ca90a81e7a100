"""The engines built on the reference's own Simulation class
(pyphasefield.simulation.Simulation, imported through oracle/refshim with
inert stand-ins for matplotlib/meshio/tinydb): the drop-in registration a
maintainer adds inside pyphasefield/Engines.

Needs the reference checkout (PPF_REFERENCE_ROOT); skipped otherwise. The
host half (constructor, initialize_fields_and_imported_data, the
reference's save_simulation / load_simulation, and the refusal to run
without a GPU) runs on CPU; the device half is marked gpu and also needs the
checkout, which machines without it cannot provide.
"""
import numpy as np
import pytest

from oracle import refshim
from tests.helpers import rel_l2

pytestmark = pytest.mark.skipif(not refshim.available(), reason="reference checkout absent")


@pytest.fixture(scope="module")
def ref_engines():
    refshim.modules()
    import sys
    from pyphasefield_gb300 import make_engines
    return make_engines(sys.modules["pyphasefield.simulation"].Simulation)


def _seeded(shape, seed=0):
    rng = np.random.default_rng(seed)
    phi0 = np.ones(shape)
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    phi0[(yy - shape[0] / 2 + 0.5) ** 2 + (xx - shape[1] / 2 + 0.5) ** 2 < 36] = 0.0
    c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    return phi0, c0


def test_host_half_on_the_reference_base(ref_engines, tmp_path):
    import sys
    base = sys.modules["pyphasefield.simulation"].Simulation
    W = ref_engines["Warren1995GB300"]
    assert issubclass(W, base)
    sim = W(dimensions=[40, 50], dx=4.6e-8, boundary_conditions="NEUMANN",
            save_path=str(tmp_path), user_data={"seed": 1})
    sim.initialize_fields_and_imported_data()  # the reference's own method
    assert [f.name for f in sim.fields] == ["phi", "c"]
    assert sim.fields[0].data.shape == (42, 52)
    # the reference's save_simulation / load_simulation read and write our state
    sim.time_step_counter = 7
    sim.save_simulation()
    again = W(dimensions=[40, 50], dx=4.6e-8, boundary_conditions="NEUMANN",
              user_data={"seed": 1})
    again.load_simulation(file_path=str(tmp_path / "step_7.npz"))
    assert again.time_step_counter == 7
    np.testing.assert_array_equal(again.fields[1].get_cells(), sim.fields[1].get_cells())
    # no CPU fallback: without a GPU the engine refuses to step
    import torch
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError, match="CUDA"):
            sim.simulate(2)


@pytest.mark.gpu
def test_device_half_on_the_reference_base(ref_engines, cuda, tmp_path):
    from oracle import restate
    W = ref_engines["Warren1995GB300"]
    shape = (48, 40)
    phi0, c0 = _seeded(shape, 3)
    sim = W(dimensions=list(shape), dx=4.6e-8, boundary_conditions="NEUMANN",
            save_path=str(tmp_path), autosave=True, autosave_rate=10,
            user_data={"seed": 5, "graph_chunk": 4})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = phi0
    sim.fields[1].data[1:-1, 1:-1] = c0
    sim.simulate(20)
    params = {k: sim.user_data[k] for k in restate.WARREN_DEFAULTS}
    ref = restate.run_warren(phi0, c0, 20, "NEUMANN", 4.6e-8, params, seed=5)
    sim.retrieve_fields_from_GPU()
    for f in (0, 1):
        assert rel_l2(sim.fields[f].get_cells(), ref[f]) < 1e-5
    assert sorted(p.name for p in tmp_path.glob("*.npz")) == ["step_10.npz", "step_20.npz"]
    back = W(dimensions=list(shape), dx=4.6e-8, boundary_conditions="NEUMANN",
             user_data={"seed": 5})
    back.load_simulation(file_path=str(tmp_path / "step_10.npz"))
    back.simulate(10)
    back.retrieve_fields_from_GPU()
    for f in (0, 1):
        assert rel_l2(back.fields[f].get_cells(), ref[f]) < 1e-5

    CH = ref_engines["CahnHilliardGB300"]
    rng = np.random.default_rng(2)
    u0 = 0.5 + rng.uniform(-0.05, 0.05, (12, 14, 10))
    ch = CH(dimensions=[12, 14, 10], dx=1.0, dt=0.01, boundary_conditions="PERIODIC",
            user_data={"M": 1.0, "epsilon": 1.0, "graph_chunk": 4})
    ch.initialize_fields_and_imported_data()
    ch.fields[0].data[1:-1, 1:-1, 1:-1] = u0
    ch.simulate(12)
    ch.retrieve_fields_from_GPU()
    want = restate.run_single("cahn_hilliard", u0, 12, "PERIODIC", 1.0, 0.01, M=1.0, epsilon=1.0)
    assert rel_l2(ch.fields[0].get_cells(), want) < 1e-5
