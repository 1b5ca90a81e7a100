"""The benchmarked workload itself against the FP64 oracle: Warren1995 on
1024 x 1024 cells from bench.py's own initial_fields() (solid disk of radius
5 centred on cell (512, 512), c = 0.40783 + U(-1e-3, 1e-3) from seed 0,
no-flux boundaries, engine defaults, dx = 4.6e-8 m), 1000 steps through
Warren1995GB300, in float64 and float32, with the noise off (alpha = 0, the
parity run) and on (alpha = 0.3 with the shared Philox stream, the timed
run).

The checker is the C restatement of the oracle (oracle/coracle.py, pinned
to the numpy restatement of Engines/Warren1995.py:50-92 in
tests/test_oracle.py); the numpy one would take minutes per run here.
Tolerances (relative L2 over the interior): float64 1e-12, float32 1e-5.
"""
import numpy as np
import pytest

import bench
from oracle import coracle, restate
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

STEPS = 1000


@pytest.fixture(scope="module")
def oracle_runs():
    phi0, c0 = bench.initial_fields()
    out = {}
    for alpha in (0.0, 0.3):
        p = dict(restate.WARREN_DEFAULTS, alpha=alpha)
        out[alpha] = coracle.run_warren(phi0, c0, STEPS, "NEUMANN", bench.DX, p, seed=bench.SEED)
    return phi0, c0, out


@pytest.mark.parametrize("alpha", [0.0, 0.3])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_benchmark_workload_matches_oracle(cuda, oracle_runs, alpha, precision, tol):
    from pyphasefield_gb300 import Warren1995GB300
    phi0, c0, ref = oracle_runs
    sim = Warren1995GB300(dimensions=list(bench.SHAPE), dx=bench.DX,
                          boundary_conditions="NEUMANN",
                          user_data={"seed": bench.SEED, "alpha": alpha, "precision": precision,
                                     "graph_chunk": 500})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = phi0
    sim.fields[1].data[1:-1, 1:-1] = c0
    sim.simulate(STEPS)
    sim.retrieve_fields_from_GPU()
    ref_phi, ref_c = ref[alpha]
    phi, c = sim.fields[0].get_cells(), sim.fields[1].get_cells()
    e_phi, e_c = rel_l2(phi, ref_phi), rel_l2(c, ref_c)
    linf = float(np.abs(phi - ref_phi).max()), float(np.abs(c - ref_c).max())
    print(f"\n{precision} alpha={alpha}: phi rel L2 {e_phi:.3e} Linf {linf[0]:.3e}; "
          f"c rel L2 {e_c:.3e} Linf {linf[1]:.3e}")
    assert e_phi < tol and e_c < tol, (e_phi, e_c, linf)
    # the crystal has grown: the comparison is not of two unchanged fields
    assert (ref_phi < 0.5).sum() > 10 * (phi0 < 0.5).sum()
