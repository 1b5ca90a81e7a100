"""CUDA kernels through the C-ABI against the oracle.

Tolerances (relative L2 over interior cells):
  * fp64 kernels vs the FP64 oracle: <= 1e-12 (rounding-order differences only);
  * fp32 kernels vs the FP64 oracle: <= 1e-5 (the precision target), with a
    per-case bound where the dynamics amplify rounding.
Bit-exact checks: temporal depth k vs k single steps, PDL on/off, tile
shapes, and exact float mass conservation of the quantised Cahn-Hilliard step.
"""
import numpy as np
import pytest

from oracle import restate
from tests.helpers import (load_golden, golden_names, rel_l2, run_single_gpu,
                           run_warren_gpu)

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 1e-5


@pytest.mark.parametrize("name", golden_names("diffusion") + golden_names("allen_cahn")
                         + golden_names("cahn_hilliard"))
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_single_field_golden(cuda, name, precision):
    d = load_golden(name)
    m = d["meta"]
    out = run_single_gpu(m["model"], d["c0"], m["steps"], m["bc"], m["dx"], m["dt"],
                         values=m["values"], precision=precision, **m["params"])
    tol = F64_TOL if precision == "fp64" else F32_TOL
    assert rel_l2(out, d["out"]) < tol


@pytest.mark.parametrize("name", golden_names("warren"))
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_warren_golden(cuda, name, precision):
    d = load_golden(name)
    m = d["meta"]
    phi, c = run_warren_gpu(d["phi0"], d["c0"], m["steps"], m["bc"], m["dx"], m["params"],
                            seed=m["seed"], precision=precision)
    tol = F64_TOL if precision == "fp64" else F32_TOL
    assert rel_l2(phi, d["phi"]) < tol
    assert rel_l2(c, d["c"]) < tol


def test_diffusion_config_256_1000_steps(cuda):
    """Diffusion 2-D 256^2, dx=1, D=1, dt=0.2, periodic, c0 = 0.5 + 0.01 N(0,1)
    (seed 0), 1000 steps: fp32 within 1e-5 of the FP64 oracle."""
    rng = np.random.default_rng(0)
    c0 = 0.5 + 0.01 * rng.standard_normal((256, 256))
    ref = restate.run_single("diffusion", c0, 1000, "PERIODIC", 1.0, 0.2, D=1.0)
    for prec, tol in (("fp32", F32_TOL), ("fp64", F64_TOL)):
        out = run_single_gpu("diffusion", c0, 1000, "PERIODIC", 1.0, 0.2, precision=prec, D=1.0)
        assert rel_l2(out, ref) < tol, prec
        assert np.abs(out - ref).max() < (1e-5 if prec == "fp32" else 1e-12)


@pytest.mark.parametrize("bc", ["PERIODIC", "NEUMANN", ["DIRCHLET", "PERIODIC"],
                                ["NEUMANN", "DIRCHLET"]])
@pytest.mark.parametrize("model", ["diffusion", "allen_cahn"])
@pytest.mark.parametrize("depth", [2, 3, 4, 8])
def test_temporal_blocking_bit_exact(cuda, model, bc, depth):
    """depth-k passes equal k single steps bit for bit (periodic wrap, no-flux
    mirror and fixed Dirichlet ghosts all stay exact inside the tile)."""
    rng = np.random.default_rng(11)
    c0 = rng.random((150, 301))
    params = dict(D=1.0) if model == "diffusion" else dict(M=0.1, epsilon=1.0, W=1.0)
    bcs = [bc] * 2 if isinstance(bc, str) else bc
    # Dirichlet faces get values; Neumann faces stay no-flux (depth > 1 needs it)
    vals = [[[0.25, 0.5] if b == "DIRCHLET" else [0.0, 0.0] for b in bcs]]
    for prec in ("fp32", "fp64"):
        a = run_single_gpu(model, c0, 16, bc, 1.0, 0.1, values=vals, precision=prec, depth=1,
                           **params)
        b = run_single_gpu(model, c0, 16, bc, 1.0, 0.1, values=vals, precision=prec,
                           depth=depth, **params)
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("depth,seg", [(4, 0), (8, 0), (2, 12), (5, 4), (7, 64)])
def test_marching_kernel_segments_bit_exact(cuda, depth, seg):
    """The marching temporal-blocking kernel (TMA-fed windows, one register
    stage per step) on a grid with interior TMA windows and edge windows,
    with the default and explicit segment lengths: depth-k passes equal k
    single steps bit for bit, and the FP64 oracle."""
    rng = np.random.default_rng(21)
    c0 = rng.random((517, 1003))
    for model, params in (("diffusion", dict(D=1.0)),
                          ("allen_cahn", dict(M=0.1, epsilon=1.0, W=1.0))):
        for bc in ("PERIODIC", ["NEUMANN", "PERIODIC"], ["DIRCHLET", "NEUMANN"]):
            bcs = [bc] * 2 if isinstance(bc, str) else bc
            vals = [[[0.25, 0.5] if b == "DIRCHLET" else [0.0, 0.0] for b in bcs]]
            for prec in ("fp32", "fp64"):
                a = run_single_gpu(model, c0, 2 * depth + 1, bc, 1.0, 0.1, values=vals,
                                   precision=prec, depth=1, **params)
                b = run_single_gpu(model, c0, 2 * depth + 1, bc, 1.0, 0.1, values=vals,
                                   precision=prec, depth=depth, tile=(0, seg) if seg else None,
                                   **params)
                np.testing.assert_array_equal(a, b)
            ref = restate.run_single(model, c0, 2 * depth + 1, bc, 1.0, 0.1, values=vals,
                                     **params)
            assert rel_l2(b, ref) < F64_TOL


@pytest.mark.parametrize("shape", [(1, 7), (7, 1), (5, 3), (33, 65), (129, 31)])
def test_odd_and_tiny_shapes(cuda, shape):
    rng = np.random.default_rng(12)
    c0 = rng.random(shape)
    for bc in ("PERIODIC", "NEUMANN", ["DIRCHLET", "NEUMANN"]):
        ref = restate.run_single("allen_cahn", c0, 6, bc, 1.0, 0.1, M=0.1, epsilon=1.0, W=1.0)
        for depth in (1, 3):
            out = run_single_gpu("allen_cahn", c0, 6, bc, 1.0, 0.1, precision="fp64",
                                 depth=depth, M=0.1, epsilon=1.0, W=1.0)
            assert rel_l2(out, ref) < F64_TOL, (bc, depth)


def test_one_dimensional_grid(cuda):
    rng = np.random.default_rng(13)
    c0 = rng.random(97)
    for bc in ("PERIODIC", "NEUMANN", "DIRCHLET"):
        ref = restate.run_single("diffusion", c0, 9, bc, 1.0, 0.3, D=1.0)
        for depth in (1, 2):
            out = run_single_gpu("diffusion", c0, 9, bc, 1.0, 0.3, precision="fp64", depth=depth,
                                 D=1.0)
            assert rel_l2(out, ref) < F64_TOL, (bc, depth)


@pytest.mark.parametrize("model", ["diffusion", "allen_cahn"])
def test_lean_2d_kernel_matches_tiled_and_oracle(cuda, model):
    """The default depth-1 kernel (warp strips of 16-byte vectors) against
    the shared-memory tile kernel (bit for bit) and the FP64 oracle, on a grid
    with interior strips, ragged right and bottom edges and every BC type."""
    rng = np.random.default_rng(15)
    c0 = rng.random((203, 517))
    params = dict(D=1.0) if model == "diffusion" else dict(M=0.1, epsilon=1.0, W=1.0)
    for bc in ("PERIODIC", "NEUMANN", ["DIRCHLET", "NEUMANN"], ["PERIODIC", "DIRCHLET"]):
        bcs = [bc] * 2 if isinstance(bc, str) else bc
        vals = [[[0.25, 0.75] if b == "DIRCHLET" else [0.0, 0.0] for b in bcs]]
        for prec in ("fp32", "fp64"):
            lean = run_single_gpu(model, c0, 7, bc, 1.0, 0.1, values=vals, precision=prec,
                                  **params)
            tiled = run_single_gpu(model, c0, 7, bc, 1.0, 0.1, values=vals, precision=prec,
                                   tile=(128, 32), **params)
            np.testing.assert_array_equal(lean, tiled)
        ref = restate.run_single(model, c0, 7, bc, 1.0, 0.1, values=vals, **params)
        assert rel_l2(lean, ref) < F64_TOL, bc


@pytest.mark.parametrize("model", ["diffusion", "allen_cahn"])
def test_lean_3d_kernel_and_z_chunks(cuda, model):
    """The default 3-D kernel (32x32 tiles, register z-window) against the
    generic tile kernel and the FP64 oracle on a grid with interior tiles,
    for several planes-per-CTA settings (results identical bit for bit)."""
    rng = np.random.default_rng(16)
    c0 = rng.random((45, 70, 101))
    params = dict(D=1.0) if model == "diffusion" else dict(M=0.1, epsilon=1.0, W=1.0)
    for bc in ("PERIODIC", ["NEUMANN", "PERIODIC", "DIRCHLET"]):
        outs = [run_single_gpu(model, c0, 4, bc, 1.0, 0.05, precision="fp64", zchunk=z, **params)
                for z in (0, 1, 7, 12, 64)]
        outs.append(run_single_gpu(model, c0, 4, bc, 1.0, 0.05, precision="fp64",
                                   tile=(64, 16), **params))
        for o in outs[1:]:
            np.testing.assert_array_equal(o, outs[0])
        ref = restate.run_single(model, c0, 4, bc, 1.0, 0.05, **params)
        assert rel_l2(outs[0], ref) < F64_TOL, bc


@pytest.mark.parametrize("shape", [(5, 6, 7), (17, 3, 40), (1, 9, 70)])
@pytest.mark.parametrize("model", ["diffusion", "allen_cahn"])
def test_three_d_single_field(cuda, shape, model):
    rng = np.random.default_rng(14)
    c0 = rng.random(shape)
    params = dict(D=1.0) if model == "diffusion" else dict(M=0.1, epsilon=1.0, W=1.0)
    for bc in ("PERIODIC", "NEUMANN", ["DIRCHLET", "PERIODIC", "NEUMANN"]):
        ref = restate.run_single(model, c0, 5, bc, 1.0, 0.05, **params)
        out = run_single_gpu(model, c0, 5, bc, 1.0, 0.05, precision="fp64", **params)
        assert rel_l2(out, ref) < F64_TOL, bc


@pytest.mark.parametrize("shape,bc", [((12, 13, 14), "PERIODIC"), ((9, 20, 7), "NEUMANN"),
                                      ((40, 37), "PERIODIC"), ((16, 24), "NEUMANN"),
                                      ((70, 3, 5), ["NEUMANN", "PERIODIC", "NEUMANN"])])
def test_cahn_hilliard_vs_oracle(cuda, shape, bc):
    rng = np.random.default_rng(15)
    c0 = 0.5 + rng.uniform(-0.05, 0.05, shape)
    ref = restate.run_single("cahn_hilliard", c0, 20, bc, 1.0, 0.01, M=1.0, epsilon=1.0)
    out = run_single_gpu("cahn_hilliard", c0, 20, bc, 1.0, 0.01, precision="fp64", M=1.0,
                         epsilon=1.0)
    assert rel_l2(out, ref) < F64_TOL
    out = run_single_gpu("cahn_hilliard", c0, 20, bc, 1.0, 0.01, precision="fp64", M=1.0,
                         epsilon=1.0, centered=1)
    assert rel_l2(out, ref) < F64_TOL


@pytest.mark.parametrize("shape,bc", [((30, 37, 45), "PERIODIC"), ((24, 100, 100), "PERIODIC"),
                                      ((26, 41, 35), "NEUMANN"),
                                      ((25, 70, 99), ["PERIODIC", "NEUMANN", "PERIODIC"])])
def test_cahn_hilliard_edge_and_interior_tiles(cuda, shape, bc):
    """Grids with partial 32 x 32 tiles, interior tiles beside edge tiles
    (whose cells outside the grid are fetched a plane ahead) and several
    z chunks: fp64 against the oracle, and the quantised float path within
    the float tolerance with its sum exactly constant."""
    q = 2.0 ** -24
    rng = np.random.default_rng(18)
    c0 = 0.5 + rng.uniform(-0.05, 0.05, shape)
    c0 = 0.5 + np.rint((c0 - 0.5) / q) * q
    ref = restate.run_single("cahn_hilliard", c0, 12, bc, 1.0, 0.01, M=1.0, epsilon=1.0)
    out = run_single_gpu("cahn_hilliard", c0, 12, bc, 1.0, 0.01, precision="fp64", M=1.0,
                         epsilon=1.0)
    assert rel_l2(out, ref) < F64_TOL
    out = run_single_gpu("cahn_hilliard", c0, 12, bc, 1.0, 0.01, precision="fp32", quantum=q,
                         centered=1, M=1.0, epsilon=1.0)
    assert rel_l2(out, ref) < F32_TOL
    assert (out - 0.5).sum() == (c0 - 0.5).sum()


def test_cahn_hilliard_quantised_conserves_mass_exactly(cuda):
    """Centered storage + 2^-24 face-flux quantum: the float field's sum is
    exactly constant, and the field stays within 1e-5 of FP64."""
    q = 2.0 ** -24
    rng = np.random.default_rng(16)
    c0 = 0.5 + rng.uniform(-0.05, 0.05, (32, 32, 32))
    c0 = 0.5 + np.rint((c0 - 0.5) / q) * q
    ref = restate.run_single("cahn_hilliard", c0, 200, "PERIODIC", 1.0, 0.01, M=1.0,
                             epsilon=1.0)
    out = run_single_gpu("cahn_hilliard", c0, 200, "PERIODIC", 1.0, 0.01, precision="fp32",
                         quantum=q, centered=1, M=1.0, epsilon=1.0)
    assert rel_l2(out, ref) < F32_TOL
    assert (out - 0.5).sum() == (c0 - 0.5).sum()
    # planes per CTA along z change only the work split, not one bit
    for zc in (1, 5, 32):
        o2 = run_single_gpu("cahn_hilliard", c0, 20, "PERIODIC", 1.0, 0.01, precision="fp32",
                            quantum=q, centered=1, zchunk=zc, M=1.0, epsilon=1.0)
        o1 = run_single_gpu("cahn_hilliard", c0, 20, "PERIODIC", 1.0, 0.01, precision="fp32",
                            quantum=q, centered=1, M=1.0, epsilon=1.0)
        np.testing.assert_array_equal(o1, o2)


def test_warren_vs_oracle_noise_and_edges(cuda):
    rng = np.random.default_rng(17)
    shape = (45, 70)
    phi0 = np.ones(shape)
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    # half-integer seed centres: no cell on a centre of symmetry (see the
    # golden generator for why such cells are excluded from fp32 parity)
    phi0[(yy - 3.5) ** 2 + (xx - 60.5) ** 2 < 49] = 0.0
    phi0[(yy - 30.5) ** 2 + (xx - 20.5) ** 2 < 36] = 0.0
    c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    p = dict(restate.WARREN_DEFAULTS, alpha=0.3)
    for bc in ("NEUMANN", "PERIODIC", ["PERIODIC", "NEUMANN"]):
        ref = restate.run_warren(phi0, c0, 12, bc, 4.6e-8, p, seed=99, step0=5)
        for prec, tol in (("fp64", F64_TOL), ("fp32", F32_TOL)):
            phi, c = run_warren_gpu(phi0, c0, 12, bc, 4.6e-8, p, seed=99, step0=5,
                                    precision=prec)
            assert rel_l2(phi, ref[0]) < tol, (bc, prec)
            assert rel_l2(c, ref[1]) < tol, (bc, prec)


@pytest.mark.parametrize("shape", [(130, 97), (64, 64), (33, 5)])
def test_warren_pdl_bit_exact(cuda, shape):
    rng = np.random.default_rng(18)
    phi0 = (rng.random(shape) > 0.7).astype(float)
    c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    p = dict(restate.WARREN_DEFAULTS, alpha=0.3)
    a = run_warren_gpu(phi0, c0, 6, "NEUMANN", 4.6e-8, p, seed=1, precision="fp32")
    b = run_warren_gpu(phi0, c0, 6, "NEUMANN", 4.6e-8, p, seed=1, precision="fp32", pdl=True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_bounded_wait_reports_timeout(cuda):
    """A barrier wait that can never complete gives up after its poll limit
    and reports PPF_STATUS_TIMEOUT; the context stays usable."""
    import ctypes as C
    import torch
    from pyphasefield_gb300 import _lib as L
    st = C.c_int32()
    L.call("ppf_status_take", C.byref(st))
    L.call("ppf_selftest_wait_timeout", 1000, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    L.call("ppf_status_take", C.byref(st))
    assert st.value & L.PPF_STATUS_TIMEOUT
    L.call("ppf_status_take", C.byref(st))
    assert st.value == 0
    # the device still runs kernels normally afterwards
    out = run_single_gpu("diffusion", np.ones((8, 8)), 2, "PERIODIC", 1.0, 0.1, D=1.0)
    np.testing.assert_array_equal(out, np.ones((8, 8)))


def test_no_timeouts_recorded(cuda):
    """The 3-D kernels' TMA waits never hit their limit in normal runs."""
    import ctypes as C
    from pyphasefield_gb300 import _lib as L
    st = C.c_int32()
    L.call("ppf_status_take", C.byref(st))
    rng = np.random.default_rng(19)
    run_single_gpu("diffusion", rng.random((40, 30, 20)), 4, "PERIODIC", 1.0, 0.05, D=1.0)
    run_single_gpu("cahn_hilliard", 0.5 + rng.uniform(-0.05, 0.05, (40, 30, 20)), 4, "NEUMANN",
                   1.0, 0.01, M=1.0, epsilon=1.0)
    L.call("ppf_status_take", C.byref(st))
    assert st.value == 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_warren_bulk_shortcut_bit_exact_and_rows(cuda, precision):
    """The exact reduced form on bulk rows (phi exactly 1 or 0 around every
    cell) changes nothing, bit for bit, for every rows-per-warp choice; the
    rows-per-warp choices agree to rounding (each is its own compiled kernel,
    so multiply-add contraction may differ)."""
    rng = np.random.default_rng(23)
    shape = (150, 200)
    phi0 = np.ones(shape)
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    phi0[(yy - 60.5) ** 2 + (xx - 100.5) ** 2 < 100] = 0.0   # solid seed (phi = 0 bulk inside)
    phi0[(yy - 20.5) ** 2 + (xx - 170.5) ** 2 < 16] = 0.3
    c0 = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    p = dict(restate.WARREN_DEFAULTS, alpha=0.3)
    ref = None
    for rows in (2, 4, 8, 16):
        full = run_warren_gpu(phi0, c0, 20, "NEUMANN", 4.6e-8, p, seed=5, precision=precision,
                              tile=(0, rows), full_eval=True)
        got = run_warren_gpu(phi0, c0, 20, "NEUMANN", 4.6e-8, p, seed=5, precision=precision,
                             tile=(0, rows))
        np.testing.assert_array_equal(got[0], full[0])
        np.testing.assert_array_equal(got[1], full[1])
        if ref is None:
            ref = full
        tol = 1e-13 if precision == "fp64" else 1e-6
        assert rel_l2(full[0], ref[0]) < tol and rel_l2(full[1], ref[1]) < tol
