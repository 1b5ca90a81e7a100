"""The batched ensemble (many engines stepped together: one launch per step,
or for four- and eight-row bands one persistent cooperative launch per chunk
of steps) and the autotuner, on the GPU. Ensemble members must match the same engines
stepped one by one (fp32: within 1e-6 relative L2; the ensemble's Allen-Cahn
band is a different kernel from the single-grid one, so rounding may differ)
and the FP64 oracle (1e-5)."""
import numpy as np
import pytest

from oracle import restate
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def _members(seed=1):
    from pyphasefield_gb300.ensemble import make_config_ensemble
    return make_config_ensemble(n=5, seed=seed, side_range=(40, 150), graph_chunk=8)


def _snapshot(sims):
    return [[f.get_cells().copy() for f in s.fields] for s in sims]


@pytest.mark.parametrize("rows,bands,persistent", [
    (2, 4, False), (4, 1, True), (8, 4, True), (2, 1, False), (2, 8, False), (2, 16, False),
    (4, 4, False), (8, 1, False), (8, 4, False)])
def test_ensemble_matches_members_stepped_alone(cuda, rows, bands, persistent):
    from pyphasefield_gb300.ensemble import Ensemble
    a = _members()
    b = _members()
    for s in b:
        s.user_data["tile"] = (0, rows)
    ens = Ensemble(a, rows=rows, bands=bands, graph_chunk=8, persistent=persistent)
    ens.simulate(40)
    ens.retrieve_fields_from_GPU()
    for s in b:
        s.simulate(40)
        s.retrieve_fields_from_GPU()
    for sa, sb in zip(a, b):
        assert sa.time_step_counter == sb.time_step_counter == 40
        for fa, fb in zip(sa.fields, sb.fields):
            assert rel_l2(fa.get_cells(), fb.get_cells()) < 1e-6


def test_ensemble_graph_equals_eager_and_oracle(cuda):
    from pyphasefield_gb300.ensemble import Ensemble
    a = _members(2)
    init = _snapshot(a)
    b = _members(2)
    Ensemble(a, rows=2, graph_chunk=4).simulate(24)
    eb = Ensemble(b, rows=2, graph_chunk=4)
    for _ in range(24):
        eb.simulate(1, use_graph=False)
    for sa, sb in zip(a, b):
        sa.retrieve_fields_from_GPU()
        sb.retrieve_fields_from_GPU()
        for fa, fb in zip(sa.fields, sb.fields):
            np.testing.assert_array_equal(fa.get_cells(), fb.get_cells())
    # member 0 is Warren1995, member 1 Allen-Cahn: against the FP64 oracle
    w = a[0]
    params = {k: w.user_data[k] for k in restate.WARREN_DEFAULTS}
    ref = restate.run_warren(init[0][0], init[0][1], 24, "NEUMANN", w.dx, params,
                             seed=w.user_data["seed"])
    assert rel_l2(w.fields[0].get_cells(), ref[0]) < 1e-5
    assert rel_l2(w.fields[1].get_cells(), ref[1]) < 1e-5
    ac = a[1]
    ref = restate.run_single("allen_cahn", init[1][0], 24, "NEUMANN", 1.0, 0.1, M=0.1,
                             epsilon=1.0, W=1.0)
    assert rel_l2(ac.fields[0].get_cells(), ref) < 1e-5


def test_config_ensemble_shape():
    from pyphasefield_gb300.ensemble import make_config_ensemble
    sims = make_config_ensemble(n=64, seed=0)
    sides = [s.dimensions[0] for s in sims]
    assert len(sims) == 64 and min(sides) >= 128 and max(sides) <= 1024
    cells = sum(s * s for s in sides)
    assert 0.5e7 < cells < 4e7


def test_autotune_picks_and_caches(cuda, tmp_path, monkeypatch):
    import json
    from pyphasefield_gb300 import DiffusionGB300
    monkeypatch.setenv("PPF_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(0)
    c0 = rng.random((512, 512))
    sim = DiffusionGB300(dimensions=[512, 512], dx=1.0, dt=0.2, boundary_conditions="PERIODIC",
                         user_data={"D": 1.0, "autotune": True, "graph_chunk": 8})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = c0
    sim.simulate(16)
    sim.retrieve_fields_from_GPU()
    cache = json.loads((tmp_path / "tune.json").read_text())
    assert len(cache) == 1
    entry = next(iter(cache.values()))
    assert entry["config"]["temporal_depth"] == sim.user_data["temporal_depth"]
    from pyphasefield_gb300.engines.models import _stencil_candidates
    assert len(entry["tried"]) == len(_stencil_candidates(sim)) == 26
    ref = restate.run_single("diffusion", c0, 16, "PERIODIC", 1.0, 0.2, D=1.0)
    assert rel_l2(sim.fields[0].get_cells(), ref) < 1e-5  # tuning did not change the state


def test_persistent_chunks_equal_single_steps(cuda):
    """One cooperative launch of 7 steps (grid barrier between steps) equals
    7 one-step launches bit for bit, on an ensemble large enough that the
    launch has many CTAs."""
    from pyphasefield_gb300.ensemble import Ensemble, make_config_ensemble
    a = make_config_ensemble(n=8, seed=4, side_range=(100, 400))
    b = make_config_ensemble(n=8, seed=4, side_range=(100, 400))
    ea = Ensemble(a, rows=2, graph_chunk=8)
    ea.simulate(7, use_graph=False)  # one persistent launch
    eb = Ensemble(b, rows=2, graph_chunk=8)
    for _ in range(7):
        eb.simulate(1, use_graph=False)
    ea.retrieve_fields_from_GPU()
    eb.retrieve_fields_from_GPU()
    for sa, sb in zip(a, b):
        for fa, fb in zip(sa.fields, sb.fields):
            np.testing.assert_array_equal(fa.get_cells(), fb.get_cells())


@pytest.mark.parametrize("rows,bands", [(4, 4), (8, 1)])
def test_persistent_equals_per_step_launches(cuda, rows, bands):
    """Four- and eight-row plans: the persistent cooperative launch (grid
    barrier between steps) and one launch per step give the same fields bit
    for bit, graph-launched chunks included."""
    from pyphasefield_gb300.ensemble import Ensemble, make_config_ensemble
    runs = []
    for persistent in (True, False):
        sims = make_config_ensemble(n=8, seed=4, side_range=(100, 400))
        ens = Ensemble(sims, rows=rows, bands=bands, graph_chunk=6, persistent=persistent)
        ens.simulate(7, use_graph=False)
        ens.simulate(12)
        ens.retrieve_fields_from_GPU()
        runs.append(_snapshot(sims))
    for ma, mb in zip(*runs):
        for fa, fb in zip(ma, mb):
            np.testing.assert_array_equal(fa, fb)


def test_ensemble_follows_parameter_edits(cuda):
    """A member's T changed between simulate() calls: the graph-launched
    ensemble equals eager launches bit for bit (no stale plan)."""
    from pyphasefield_gb300.ensemble import Ensemble
    runs = []
    for use_graph in (True, False):
        sims = _members(3)
        ens = Ensemble(sims, rows=2, graph_chunk=4, use_graph=use_graph)
        ens.simulate(12)
        sims[0].user_data["T"] -= 10.0
        ens.simulate(12)
        ens.retrieve_fields_from_GPU()
        runs.append(_snapshot(sims))
    for ma, mb in zip(*runs):
        for fa, fb in zip(ma, mb):
            np.testing.assert_array_equal(fa, fb)


def test_ensemble_rows_autotuned_and_cached(cuda, tmp_path, monkeypatch):
    import json
    from pyphasefield_gb300.ensemble import Ensemble
    monkeypatch.setenv("PPF_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    sims = _members(5)
    init = _snapshot(sims)
    ens = Ensemble(sims, graph_chunk=4)
    assert ens.rows in (2, 4, 8) and ens.bands in (1, 4)
    assert ens.persistent in (True, False) and (ens.rows != 2 or not ens.persistent)
    cache = json.loads((tmp_path / "tune.json").read_text())
    entry = next(iter(cache.values()))
    assert entry["config"] == {"rows": ens.rows, "bands": ens.bands, "persistent": ens.persistent}
    assert len(entry["tried"]) == 10
    # tuning ran on scratch copies: the members still hold their initial
    # (float32-rounded) state
    ens.retrieve_fields_from_GPU()
    for m, s in zip(init, sims):
        for f0, f in zip(m, s.fields):
            np.testing.assert_array_equal(f0.astype(np.float32), f.get_cells())
    # a second ensemble of the same mix takes the cached choice
    again = Ensemble(_members(5), graph_chunk=4)
    assert (again.rows, again.bands, again.persistent) == (ens.rows, ens.bands, ens.persistent)
