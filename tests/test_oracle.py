"""The oracle itself: pinned to pyphasefield's own engine functions.

* every committed golden vector (generated from the reference's numpy engines
  by tests/golden/make_golden.py) is reproduced by oracle.restate;
* where the reference checkout exists, the restatement equals the reference's
  functions on fresh inputs (bit for bit: same numpy operations);
* Philox4x32-10 matches the generator's published known-answer vectors;
* analytic checks the reference's tests lack: discrete Fourier-mode decay of
  FTCS diffusion and exact periodic mass conservation in FP64.
"""
import numpy as np
import pytest

from oracle import refshim, restate
from oracle.philox import noise_uniform, philox4x32_10
from tests.helpers import golden_names, load_golden, rel_l2


EXPLICIT_GOLDEN = [n for n in golden_names() if not n.startswith(("implicit_", "crank_nicolson_", "phase_implicit_", "ncgpu_"))]


@pytest.mark.parametrize("name", EXPLICIT_GOLDEN)
def test_restatement_reproduces_golden(name):
    d = load_golden(name)
    m = d["meta"]
    if m["model"] == "warren1995":
        phi, c = restate.run_warren(d["phi0"], d["c0"], m["steps"], m["bc"], m["dx"],
                                    m["params"], seed=m["seed"])
        assert rel_l2(phi, d["phi"]) < 1e-13
        assert rel_l2(c, d["c"]) < 1e-13
    else:
        out = restate.run_single(m["model"], d["c0"], m["steps"], m["bc"], m["dx"], m["dt"],
                                 values=m["values"], **m["params"])
        assert rel_l2(out, d["out"]) < 1e-13


needs_ref = pytest.mark.skipif(not refshim.available(), reason="reference checkout absent")


@needs_ref
@pytest.mark.parametrize("bc", ["PERIODIC", "NEUMANN", ["DIRCHLET", "PERIODIC"]])
@pytest.mark.parametrize("model", ["diffusion", "allen_cahn"])
def test_restatement_equals_reference_engines(model, bc):
    rng = np.random.default_rng(5)
    c0 = rng.random((11, 13))
    params = dict(D=0.7) if model == "diffusion" else dict(M=0.1, epsilon=1.0, W=1.0)
    vals = [[[0.2, 0.3], [0.1, -0.1]]]
    a = refshim.run_single(model, c0, 4, bc, 1.0, 0.1, values=vals, **params)
    b = restate.run_single(model, c0, 4, bc, 1.0, 0.1, values=vals, **params)
    np.testing.assert_array_equal(a, b)


@needs_ref
@pytest.mark.parametrize("bc", ["PERIODIC", "NEUMANN"])
def test_cahn_hilliard_restatement_equals_reference(bc):
    rng = np.random.default_rng(6)
    c0 = 0.5 + rng.uniform(-0.1, 0.1, (9, 10, 8))
    a = refshim.run_cahn_hilliard_extended(c0, 3, bc, 1.0, 0.01, 1.0, 1.0)
    b = restate.run_single("cahn_hilliard", c0, 3, bc, 1.0, 0.01, M=1.0, epsilon=1.0)
    np.testing.assert_array_equal(a, b)


@needs_ref
def test_warren_restatement_equals_reference_with_noise():
    rng = np.random.default_rng(7)
    n = (20, 18)
    phi0 = np.ones(n)
    phi0[8:12, 7:11] = 0.0
    c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, n)
    p = dict(restate.WARREN_DEFAULTS)
    noise = [noise_uniform(3, s, n) for s in range(3)]
    a = refshim.run_warren(phi0, c0, 3, ["PERIODIC", "NEUMANN"], 4.6e-8, p, noise=noise)
    b = restate.run_warren(phi0, c0, 3, ["PERIODIC", "NEUMANN"], 4.6e-8, p, seed=3)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_philox_known_answers():
    kat = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
           ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in kat:
        assert tuple(int(v) for v in philox4x32_10(ctr, key)) == want


def test_noise_uniform_range_and_independence():
    u = noise_uniform(0, 0, (64, 64))
    assert u.min() >= 0 and u.max() < 1
    assert abs(u.mean() - 0.5) < 0.02
    assert not np.array_equal(u, noise_uniform(0, 1, (64, 64)))
    assert not np.array_equal(u, noise_uniform(1, 0, (64, 64)))
    np.testing.assert_array_equal(u * 2 ** 24, np.floor(u * 2 ** 24))


@pytest.mark.parametrize("shape,k", [((64,), 3), ((32, 48), 5), ((16, 12, 20), 2)])
def test_ftcs_fourier_mode_decay(shape, k):
    """A periodic Fourier mode decays by exactly prod(1 - 4r sin^2(pi k/N))
    per step under the FTCS update (r = D dt/dx^2)."""
    D, dt, dx = 1.0, 0.1, 1.0
    r = D * dt / dx ** 2
    grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    mode = np.ones(shape)
    factor = 1.0
    for a, n in enumerate(shape):
        mode = mode * np.cos(2 * np.pi * k * grids[a] / n)
        factor += -4 * r * np.sin(np.pi * k / n) ** 2
    steps = 7
    out = restate.run_single("diffusion", mode, steps, "PERIODIC", dx, dt, D=D)
    np.testing.assert_allclose(out, mode * factor ** steps, rtol=0, atol=1e-12)


def test_periodic_mass_conservation_fp64():
    rng = np.random.default_rng(8)
    c0 = 0.5 + rng.uniform(-0.05, 0.05, (12, 12, 12))
    out = restate.run_single("cahn_hilliard", c0, 20, "PERIODIC", 1.0, 0.01, M=1.0, epsilon=1.0)
    assert abs(out.sum() - c0.sum()) / c0.sum() < 1e-13
    out = restate.run_single("diffusion", c0, 20, "NEUMANN", 1.0, 0.1, D=1.0)
    assert abs(out.sum() - c0.sum()) / c0.sum() < 1e-13


def test_allen_cahn_flat_interface_is_stationary():
    """The profile phi = (1 + tanh(x / (2 delta)))/2 with
    delta = eps / sqrt(32 W) is a stationary solution of the continuous
    Allen-Cahn equation phi_t = M(eps^2 phi_xx - 16 W g'(phi)); the discrete
    update moves it only by the O(dx^2) truncation error."""
    eps, W, M = 16.0, 1.0, 0.1  # interface width 2 delta ~ 5.7 cells
    delta = eps / np.sqrt(32 * W)
    x = np.arange(128) - 63.5
    prof = 0.5 * (1 + np.tanh(x / (2 * delta)))
    phi0 = np.tile(prof, (4, 1))
    out = restate.run_single("allen_cahn", phi0, 500, ["PERIODIC", "NEUMANN"], 1.0, 0.002,
                             M=M, epsilon=eps, W=W)
    assert np.abs(out - phi0).max() < 2e-3


@pytest.mark.parametrize("shape,bc,alpha,steps", [
    ((40, 52), "NEUMANN", 0.0, 30),
    ((33, 47), ["PERIODIC", "NEUMANN"], 0.3, 40),
    ((64, 64), "PERIODIC", 0.3, 60),
    ((21, 30), ["NEUMANN", "DIRCHLET"], 0.3, 12),
])
def test_c_restatement_equals_numpy_restatement(shape, bc, alpha, steps):
    """oracle/warren_c.c (the checker for the full-size Warren1995 runs) against
    the numpy restatement: equal up to the last bits of atan2/cos/sin."""
    from oracle import coracle
    rng = np.random.default_rng(11)
    phi0 = np.ones(shape)
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    phi0[(yy - shape[0] // 2) ** 2 + (xx - shape[1] // 2) ** 2 < 25] = 0.0
    c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    p = dict(restate.WARREN_DEFAULTS, alpha=alpha)
    vals = [[[0.0, 0.0], [0.9, 1.0]], [[0.0, 0.0], [0.41, 0.40]]] if "DIRCHLET" in bc else None
    a = restate.run_warren(phi0, c0, steps, bc, 4.6e-8, p, seed=5, step0=3, values=vals)
    b = coracle.run_warren(phi0, c0, steps, bc, 4.6e-8, p, seed=5, step0=3, values=vals)
    for x, y in zip(a, b):
        assert rel_l2(y, x) < 1e-14
        assert np.abs(x - y).max() < 1e-13
