"""FP64 diagnostics (mass and free energy) of FP32/FP64 fields through the
C-ABI, against numpy in double. Tolerance: 1e-12 relative (both sides sum
the same float64 values; only the summation order differs)."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import make_structs, to_dev

pytestmark = pytest.mark.gpu


def _scratch(grid):
    import torch
    from pyphasefield_gb300 import _lib as L
    n = C.c_size_t()
    L.call("ppf_reduce_scratch_bytes", C.byref(grid), C.byref(n))
    return torch.empty(max(n.value, 8), dtype=torch.uint8, device="cuda"), n.value


def energy_numpy(x, bc, dx, w, kappa):
    """dx^d * sum[w x^2 (1-x)^2 + kappa/2 sum_axes ((x_{+1} - x)/dx)^2], the
    +1 neighbour taken with the boundary rule (periodic wrap, no-flux mirror,
    Dirichlet value 0)."""
    x = np.asarray(x, dtype=np.float64)
    bcs = [bc] * x.ndim if isinstance(bc, str) else bc
    e = w * x ** 2 * (1 - x) ** 2
    for a, b in enumerate(bcs):
        nxt = np.roll(x, -1, a)
        last = [slice(None)] * x.ndim
        last[a] = -1
        last = tuple(last)
        if b == "NEUMANN":
            nxt[last] = x[last]
        elif b == "DIRCHLET":
            nxt[last] = 0.0
        e = e + 0.5 * kappa * ((nxt - x) / dx) ** 2
    return e.sum() * dx ** x.ndim


@pytest.mark.parametrize("shape", [(1000, 777), (3, 5), (17, 40, 33), (1, 1, 64)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_reduce_sum(cuda, shape, precision):
    import torch
    from pyphasefield_gb300 import _lib as L
    rng = np.random.default_rng(21)
    x = rng.random(shape) - 0.3
    g, b, ks, pitch = make_structs(shape, "PERIODIC")
    dtype = torch.float32 if precision == "fp32" else torch.float64
    t = to_dev(x, ks, pitch, dtype, "cuda")
    t[..., ks[-1]:] = 1e30  # padding columns must be ignored
    scratch, nbytes = _scratch(g)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    sfx = "f32" if precision == "fp32" else "f64"
    L.call(f"ppf_reduce_sum_{sfx}", C.c_void_p(t.data_ptr()), C.byref(g),
           C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()), C.c_size_t(nbytes),
           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    want = t[..., :ks[-1]].double().sum().item()
    assert abs(out.item() - want) <= 1e-12 * abs(want)


@pytest.mark.parametrize("shape,bc", [((64, 48), "PERIODIC"), ((30, 31), "NEUMANN"),
                                      ((12, 10, 9), ["PERIODIC", "NEUMANN", "DIRCHLET"])])
def test_free_energy(cuda, shape, bc):
    import torch
    from pyphasefield_gb300 import _lib as L
    rng = np.random.default_rng(22)
    x = rng.random(shape)
    g, b, ks, pitch = make_structs(shape, bc)
    t = to_dev(x, ks, pitch, torch.float64, "cuda")
    scratch, nbytes = _scratch(g)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    L.call("ppf_free_energy_f64", C.c_void_p(t.data_ptr()), C.byref(g), C.byref(b),
           C.c_double(0.5), C.c_double(16.0), C.c_double(2.0), C.c_void_p(out.data_ptr()),
           C.c_void_p(scratch.data_ptr()), C.c_size_t(nbytes),
           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    want = energy_numpy(x, bc, 0.5, 16.0, 2.0)
    assert abs(out.item() - want) <= 1e-12 * abs(want)


def test_reduce_rejects_small_scratch(cuda):
    import torch
    from pyphasefield_gb300 import _lib as L
    g, b, ks, pitch = make_structs((100, 100), "PERIODIC")
    t = torch.zeros((100, pitch), device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    scratch = torch.empty(8, dtype=torch.uint8, device="cuda")
    with pytest.raises(L.PpfError) as e:
        L.call("ppf_reduce_sum_f32", C.c_void_p(t.data_ptr()), C.byref(g),
               C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()), C.c_size_t(8), None)
    assert e.value.code == L.PPF_ERR_INVALID


def test_check_finite_flags_nan(cuda):
    import torch
    from pyphasefield_gb300 import _lib as L
    g, b, ks, pitch = make_structs((50, 70), "PERIODIC")
    t = torch.zeros((50, pitch), device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.call("ppf_check_finite_f32", C.c_void_p(t.data_ptr()), C.byref(g), C.c_void_p(st.data_ptr()), s)
    assert st.item() == 0
    t[17, 33] = float("nan")
    L.call("ppf_check_finite_f32", C.c_void_p(t.data_ptr()), C.byref(g), C.c_void_p(st.data_ptr()), s)
    assert st.item() & L.PPF_STATUS_NONFINITE
