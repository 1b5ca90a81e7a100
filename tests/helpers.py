"""Shared helpers: golden fixtures and direct C-ABI drivers for GPU tests."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
BC = {"PERIODIC": 0, "NEUMANN": 1, "DIRCHLET": 2}


def golden_names(prefix=""):
    return sorted(p.stem for p in GOLDEN.glob(f"{prefix}*.npz"))


def load_golden(name):
    with np.load(GOLDEN / f"{name}.npz") as z:
        d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def bc_list(bc, nd):
    return [bc] * nd if isinstance(bc, str) else list(bc)


def make_structs(shape, bc, values=None, nfields=1):
    """PpfGrid (pitch = nx rounded to 32) and PpfBoundary for an interior shape."""
    from pyphasefield_gb300 import _lib as L
    nd = len(shape)
    kshape = (1,) + tuple(shape) if nd == 1 else tuple(shape)
    pitch = (kshape[-1] + 31) // 32 * 32
    g = L.PpfGrid()
    g.ndim = len(kshape)
    for i, n in enumerate(kshape):
        g.shape[i] = n
    g.pitch = pitch
    b = L.PpfBoundary()
    off = len(kshape) - nd
    if off:
        b.type[0] = 0
    for a, name in enumerate(bc_list(bc, nd)):
        b.type[a + off] = BC[name]
        if values is not None:
            for j in range(min(nfields, len(values))):
                for s in range(2):
                    b.value[j][a + off][s] = values[j][a][s]
    return g, b, kshape, pitch


def to_dev(x, kshape, pitch, dtype, device):
    import torch
    t = torch.zeros(kshape[:-1] + (pitch,), dtype=dtype, device=device)
    t[..., :kshape[-1]] = torch.from_numpy(np.asarray(x, dtype=np.float64).reshape(kshape)).to(
        device=device, dtype=dtype)
    return t


def from_dev(t, kshape, shape):
    return t[..., :kshape[-1]].double().cpu().numpy().reshape(shape)


def run_single_gpu(model, c0, steps, bc, dx, dt, values=None, precision="fp64", depth=1,
                   tile=None, pdl=False, device="cuda", quantum=0.0, centered=0, zchunk=0,
                   **params):
    """Advance a one-field model `steps` steps through the C-ABI (ping-pong)."""
    import torch
    from pyphasefield_gb300 import _lib as L
    dtype = torch.float64 if precision == "fp64" else torch.float32
    sfx = "f64" if precision == "fp64" else "f32"
    c0 = np.asarray(c0, dtype=np.float64)
    g, b, kshape, pitch = make_structs(c0.shape, bc, values)
    init = c0 - 0.5 if centered else c0
    a = to_dev(init, kshape, pitch, dtype, device)
    o = torch.zeros_like(a)
    t = L.PpfTiling()
    t.tile_x, t.tile_y = (tile if tile else (0, 0))
    t.pdl = 1 if pdl else 0
    t.zchunk = int(zchunk)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    done = 0
    while done < steps:
        k = min(depth, steps - done)
        t.depth = k
        if model == "diffusion":
            p = L.PpfDiffusionParams(dx, dt, params["D"])
            L.call(f"ppf_diffusion_step_{sfx}", C.byref(p), C.byref(g), C.byref(b),
                   C.c_void_p(a.data_ptr()), C.c_void_p(o.data_ptr()), C.byref(t), s)
        elif model == "allen_cahn":
            p = L.PpfAllenCahnParams(dx, dt, params["M"], params["epsilon"], params["W"])
            L.call(f"ppf_allen_cahn_step_{sfx}", C.byref(p), C.byref(g), C.byref(b),
                   C.c_void_p(a.data_ptr()), C.c_void_p(o.data_ptr()), C.byref(t), s)
        elif model == "cahn_hilliard":
            p = L.PpfCahnHilliardParams(dx, dt, params["M"], params["epsilon"], quantum)
            p.centered = centered
            L.call(f"ppf_cahn_hilliard_step_{sfx}", C.byref(p), C.byref(g), C.byref(b),
                   C.c_void_p(a.data_ptr()), C.c_void_p(o.data_ptr()), None, None,
                   C.byref(t), s)
        else:
            raise ValueError(model)
        a, o = o, a
        done += k
    torch.cuda.synchronize()
    out = from_dev(a, kshape, c0.shape)
    return out + 0.5 if centered else out


def warren_params_struct(params, dx):
    from oracle import restate
    from pyphasefield_gb300 import _lib as L
    p = restate.warren_derived(params, dx)
    vals = dict(p, dx=dx)
    return L.PpfWarren1995Params(*[float(vals[n]) for n in L.WARREN_PARAM_NAMES]), p


def run_warren_gpu(phi0, c0, steps, bc, dx, params, seed=0, precision="fp64", tile=None,
                   pdl=False, device="cuda", values=None, step0=0, full_eval=False):
    import torch
    from pyphasefield_gb300 import _lib as L
    dtype = torch.float64 if precision == "fp64" else torch.float32
    sfx = "f64" if precision == "fp64" else "f32"
    g, b, kshape, pitch = make_structs(np.shape(phi0), bc, values, nfields=2)
    prm, _ = warren_params_struct(params, dx)
    P = [to_dev(phi0, kshape, pitch, dtype, device), to_dev(c0, kshape, pitch, dtype, device)]
    Q = [torch.zeros_like(P[0]), torch.zeros_like(P[1])]
    t = L.PpfTiling()
    t.depth = 1
    t.tile_x, t.tile_y = (tile if tile else (0, 0))
    t.pdl = 1 if pdl else 0
    t.flags = L.PPF_TILING_FULL_EVAL if full_eval else 0
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for k in range(steps):
        L.call(f"ppf_warren1995_step_{sfx}", C.byref(prm), C.byref(g), C.byref(b),
               C.c_void_p(P[0].data_ptr()), C.c_void_p(P[1].data_ptr()),
               C.c_void_p(Q[0].data_ptr()), C.c_void_p(Q[1].data_ptr()),
               C.c_uint64(seed), C.c_uint64(step0 + k), None, C.byref(t), s)
        P, Q = Q, P
    torch.cuda.synchronize()
    return from_dev(P[0], kshape, np.shape(phi0)), from_dev(P[1], kshape, np.shape(phi0))
