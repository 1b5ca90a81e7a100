"""The allocation-free mass sum, ppf_reduce_sum_f32_noalloc.

It exists for callers that cannot allocate device memory (their memory
manager owns the GPU, or allocation is not allowed where they need the
mass): it takes no scratch and keeps its partial sums in a fixed array inside
the library. This test calls it through the C ABI twice in a row and checks
both results against ppf_reduce_sum_f32 (which takes caller scratch) and,
independently of the library's kernels, against numpy's float64 sum of the
same float32 values, at the tolerance the other reduction tests use (1e-12
relative). The file is named to run last, and it works alone in a fresh
process as well.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import make_structs, to_dev

pytestmark = pytest.mark.gpu


def _sum_with_scratch(t, g):
    import torch
    from pyphasefield_gb300 import _lib as L
    n = C.c_size_t()
    L.call("ppf_reduce_scratch_bytes", C.byref(g), C.byref(n))
    scratch = torch.empty(max(n.value, 8), dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    L.call("ppf_reduce_sum_f32", C.c_void_p(t.data_ptr()), C.byref(g), C.c_void_p(out.data_ptr()),
           C.c_void_p(scratch.data_ptr()), C.c_size_t(n.value),
           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return out.item()


@pytest.mark.parametrize("shape", [(1000, 777), (4, 3000), (33, 17, 45), (2, 700, 64)])
def test_noalloc_sum_matches_scratch_sum_twice(cuda, shape):
    import torch
    from pyphasefield_gb300 import _lib as L
    rng = np.random.default_rng(31)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    g, b, ks, pitch = make_structs(shape, "PERIODIC")
    for call in range(2):
        x = rng.random(shape) - 0.25 * call
        t = to_dev(x, ks, pitch, torch.float32, "cuda")
        want = _sum_with_scratch(t, g)
        out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        L.call("ppf_reduce_sum_f32_noalloc", C.c_void_p(t.data_ptr()), C.byref(g),
               C.c_void_p(out.data_ptr()), s)
        torch.cuda.synchronize()
        assert abs(out.item() - want) <= 1e-12 * abs(want), (call, out.item(), want)
        exact = x.astype(np.float32).astype(np.float64).sum()
        assert abs(out.item() - exact) <= 1e-12 * abs(exact), (call, out.item(), exact)


def test_noalloc_sum_rejects_bad_arguments(cuda):
    from pyphasefield_gb300 import _lib as L
    g, b, ks, pitch = make_structs((10, 10), "PERIODIC")
    with pytest.raises(L.PpfError) as e:
        L.call("ppf_reduce_sum_f32_noalloc", None, C.byref(g), None, None)
    assert e.value.code == L.PPF_ERR_INVALID
