"""The implicit / Crank-Nicolson diffusion oracle (oracle/implicit_ref.py) on
the CPU: pinned to the reference's own engine functions through the golden
fixtures, and the library's solution methods (segmented cyclic recurrences,
Chebyshev semi-iteration) restated in float64 against the dense solve."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import implicit_ref as I

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz")
               if p.stem.startswith(("implicit_", "crank_nicolson_")))


def load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    return json.loads(str(z["meta"])), z["c0"], z["out"]


def test_fixture_set_complete():
    assert len(CASES) == 11


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(name):
    meta, c0, out = load(name)
    got = I.run(c0, meta["steps"], meta["solver"], meta["D"], meta["dt"], meta["dx"], meta["adi"])
    err = np.abs(got - out).max() / np.abs(out).max()
    # the GMRES engines stop at a residual of 1e-5 relative to the right-hand side
    assert err <= (1e-4 if meta["gmres"] else 1e-13), err


@pytest.mark.parametrize("alpha", [1e-3, 0.25, 1.0, 40.0, 2000.0])
@pytest.mark.parametrize("n", [3, 4, 31, 32, 33, 255, 1000])
@pytest.mark.parametrize("seg", [32, 256])
def test_segmented_line_solve(alpha, n, seg):
    d = np.random.default_rng(n).standard_normal(n)
    ref = I.line_solve(d, alpha, 0)
    got = I.line_solve_segmented(d, alpha, seg)
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def test_recurrence_root_factorisation():
    for alpha in (1e-6, 0.3, 7.0, 1e5):
        r = I.recurrence_root(alpha)
        assert 0 < r < 1
        assert alpha * r * r - (1 + 2 * alpha) * r + alpha == pytest.approx(0, abs=1e-12 * (1 + alpha))


@pytest.mark.parametrize("shape", [(9, 11), (5, 6, 7)])
@pytest.mark.parametrize("alpha", [0.05, 1.0, 30.0])
def test_fft_and_chebyshev_match_dense(shape, alpha):
    rng = np.random.default_rng(3)
    b = rng.random(shape)
    dense = I.full_solve_dense(b, alpha)
    np.testing.assert_allclose(I.full_solve_fft(b, alpha), dense, rtol=0, atol=1e-13)
    cheb = I.chebyshev_solve(b, b, alpha, 1e-12)
    assert np.abs(cheb - dense).max() <= 1e-11 * np.abs(dense).max()


def test_chebyshev_bound_holds_per_iteration_count():
    # the a priori count is enough, and half of it is not
    rng = np.random.default_rng(4)
    b = rng.random((16, 12))
    alpha, tol = 5.0, 1e-9
    x = I.full_solve_fft(b, alpha)
    k, *_ = I.chebyshev_plan(alpha, 2, tol)
    assert np.abs(I.chebyshev_solve(b, b, alpha, tol) - x).max() <= tol * np.abs(b).max()
    half = I.chebyshev_plan(alpha, 2, tol ** 0.5)[0]
    assert half < k


def test_reference_degenerate_short_axes_rejected():
    with pytest.raises(ValueError):
        I.line_solve(np.ones(2), 1.0, 0)
    with pytest.raises(ValueError):
        I.full_solve_dense(np.ones((2, 5)), 1.0)


PHASE = sorted(p.stem for p in GOLDEN.glob("phase_implicit_*.npz"))


def test_phase_fixture_set_complete():
    assert len(PHASE) == 11


@pytest.mark.parametrize("name", PHASE)
def test_phase_oracle_matches_reference_fixture(name):
    z = np.load(GOLDEN / f"{name}.npz")
    m = json.loads(str(z["meta"]))
    p = m["params"]
    got = I.run_phase(m["model"], z["c0"], m["steps"], m["solver"], p["M"], p["W"],
                      p["epsilon"], m["dt"], m["dx"], m["adi"], m["gmres"])
    err = np.abs(got - z["out"]).max() / np.abs(z["out"]).max()
    assert err <= (1e-3 if m["gmres"] else 1e-13), err


def test_var_line_solve_shared_and_per_cell_diagonals():
    rng = np.random.default_rng(6)
    b = rng.random((7, 9))
    d1 = 3.0 + rng.random(9)
    x = I.var_line_solve(b, d1, 1.0, 1)
    full = np.broadcast_to(d1, b.shape)
    np.testing.assert_allclose(I.var_line_solve(b, full, 1.0, 1), x, rtol=1e-14)
    # residual of every row
    r = d1 * x - 1.0 * (np.roll(x, 1, 1) + np.roll(x, -1, 1)) - b
    assert np.abs(r).max() < 1e-13
