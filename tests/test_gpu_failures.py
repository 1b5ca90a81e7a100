"""Failure detection at the engine level, and graphs that never replay stale
parameters.

Faults are made on the host (a NaN written into a field) or by the library's
own bounded-wait self-test (a barrier nothing completes, whose wait gives up
after a few polls and reports PPF_STATUS_TIMEOUT): no test faults, traps or
hangs the GPU. The engines must raise EngineFault instead of stepping on
from a state a kernel reported as corrupt.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clear_library_status():
    from pyphasefield_gb300 import _lib as L
    v = C.c_int32()
    L.call("ppf_status_take", C.byref(v))


def _diffusion(shape=(64, 64), **ud):
    from pyphasefield_gb300 import DiffusionGB300
    rng = np.random.default_rng(0)
    sim = DiffusionGB300(dimensions=list(shape), dx=1.0, dt=0.2, boundary_conditions="PERIODIC",
                         user_data=dict({"D": 1.0, "graph_chunk": 8}, **ud))
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = 0.5 + 0.01 * rng.standard_normal(shape)
    return sim


def test_nan_on_the_device_stops_simulate_within_two_chunks(cuda):
    import torch
    from pyphasefield_gb300.engines.base import EngineFault
    _clear_library_status()
    sim = _diffusion()
    sim.simulate(16)
    sim.synchronize()
    with torch.cuda.stream(sim._ppf_stream):
        sim.device_fields()[0][3, 5] = float("nan")
    with pytest.raises(EngineFault, match="NaN or Inf"):
        sim.simulate(8 * 8)
    # raised at the third chunk boundary at the latest, not after all eight;
    # the counter covers the chunks launched before the fault
    assert 16 + 8 <= sim.time_step_counter <= 16 + 3 * 8
    # the fault was reported once: the engine's word is clear again
    sim.simulate(8)
    with pytest.raises(EngineFault):  # the field still holds the NaN
        sim.retrieve_fields_from_GPU()


def test_nan_from_the_host_is_reported_at_retrieve(cuda):
    from pyphasefield_gb300.engines.base import EngineFault
    _clear_library_status()
    sim = _diffusion(use_graph=False)
    sim.fields[0].data[10, 10] = np.inf
    sim.simulate(3)
    with pytest.raises(EngineFault, match="NaN or Inf"):
        sim.retrieve_fields_from_GPU()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_clean_runs_raise_nothing(cuda, precision):
    _clear_library_status()
    sim = _diffusion(precision=precision)
    sim.simulate(40)
    sim.retrieve_fields_from_GPU()
    assert np.isfinite(sim.fields[0].get_cells()).all()


def test_timed_out_wait_makes_the_next_simulate_raise(cuda):
    from pyphasefield_gb300 import _lib as L
    from pyphasefield_gb300.engines.base import EngineFault
    _clear_library_status()
    sim = _diffusion()
    sim.simulate(8)
    sim.synchronize()
    # a barrier wait that nothing completes gives up after 4 polls
    L.call("ppf_selftest_wait_timeout", 4, C.c_void_p(sim._ppf_stream.cuda_stream))
    with pytest.raises(EngineFault, match="timed out"):
        sim.simulate(64)
        sim.retrieve_fields_from_GPU()
    _clear_library_status()


def test_status_check_can_be_switched_off(cuda):
    _clear_library_status()
    sim = _diffusion(check_status=False)
    sim.fields[0].data[10, 10] = np.nan
    sim.simulate(16)
    sim.retrieve_fields_from_GPU()  # no sentinel: no error
    assert np.isnan(sim.fields[0].get_cells()).any()


def _warren(use_graph):
    from pyphasefield_gb300 import Warren1995GB300
    rng = np.random.default_rng(4)
    shape = (40, 50)
    phi0 = np.ones(shape)
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    phi0[(yy - 19.5) ** 2 + (xx - 24.5) ** 2 < 25] = 0.0
    sim = Warren1995GB300(dimensions=list(shape), dx=4.6e-8, boundary_conditions="NEUMANN",
                          user_data={"seed": 2, "graph_chunk": 64, "use_graph": use_graph})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = phi0
    sim.fields[1].data[1:-1, 1:-1] = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    return sim


def test_graphs_follow_user_data_edits(cuda):
    """Changing T (and alpha) between simulate() calls: the captured-graph
    run equals the eager run bit for bit, so no chunk replays old constants."""
    runs = []
    for use_graph in (True, False):
        sim = _warren(use_graph)
        sim.simulate(130)
        sim.user_data["T"] = 1560.0
        sim.simulate(130)
        sim.user_data["alpha"] = 0.0
        sim.simulate(130)
        sim.user_data["T"] = 1574.0  # back to the first parameter set
        sim.simulate(130)
        sim.retrieve_fields_from_GPU()
        runs.append([f.get_cells().copy() for f in sim.fields])
    for a, b in zip(*runs):
        np.testing.assert_array_equal(a, b)
    # and the edit did change the physics
    ref = _warren(False)
    ref.simulate(520)
    ref.retrieve_fields_from_GPU()
    assert not np.array_equal(ref.fields[0].get_cells(), runs[0][0])
