"""Device-side plumbing for the engines: the pitched interior-only layout in
HBM, host<->device transfers, and the ctypes structs passed to the library.

Layout: a field of interior shape (nz, ny, nx) (or (ny, nx); a 1-D field of
n cells is stored as (1, n)) is a torch tensor of shape (..., pitch) with
pitch = nx rounded up to 32 elements (128 bytes for float), so every row
starts 128-byte aligned and 16-byte vector loads stay aligned. No ghost
cells are stored: the library applies the boundary rule while loading tiles.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .simulation import bc_per_axis

BC_CODES = {"PERIODIC": L.PPF_BC_PERIODIC, "NEUMANN": L.PPF_BC_NEUMANN,
            "DIRCHLET": L.PPF_BC_DIRCHLET}


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 engines need a CUDA device (no CPU path exists)")
    L.load()
    return torch.device("cuda", torch.cuda.current_device())


class DeviceGrid:
    """Pitched layout of one field on the device."""

    def __init__(self, shape, dtype: torch.dtype, device: torch.device):
        shape = tuple(int(n) for n in shape)
        if not 1 <= len(shape) <= 3 or min(shape) < 1:
            raise ValueError(f"unsupported grid shape {shape}")
        self.user_shape = shape
        self.kshape = (1,) + shape if len(shape) == 1 else shape
        nx = self.kshape[-1]
        self.pitch = (nx + 31) // 32 * 32
        self.alloc_shape = self.kshape[:-1] + (self.pitch,)
        self.dtype = dtype
        self.device = device
        g = L.PpfGrid()
        g.ndim = len(self.kshape)
        g.reserved = 0
        for i, n in enumerate(self.kshape):
            g.shape[i] = n
        g.pitch = self.pitch
        self.grid = g
        self.cells = int(np.prod(shape))

    @property
    def np_dtype(self):
        return np.float32 if self.dtype == torch.float32 else np.float64

    def empty(self) -> torch.Tensor:
        return torch.zeros(self.alloc_shape, dtype=self.dtype, device=self.device)

    def view(self, t: torch.Tensor) -> torch.Tensor:
        return t[..., : self.kshape[-1]]

    def upload(self, dst: torch.Tensor, host: np.ndarray, stream: torch.cuda.Stream):
        """H2D copy of a host interior array (any float dtype) into dst
        through pinned memory, ordered on `stream`. Returns the pinned
        staging tensor (keep it alive until the stream passes the copy).
        The copy is ordered after the work already queued on the current
        stream (the zero fill of buffers allocated there)."""
        a = np.ascontiguousarray(np.asarray(host).astype(self.np_dtype).reshape(self.kshape))
        pinned = torch.from_numpy(a).pin_memory()
        stream.wait_stream(torch.cuda.current_stream(dst.device))
        with torch.cuda.stream(stream):
            self.view(dst).copy_(pinned, non_blocking=True)
        return pinned

    def download(self, src: torch.Tensor, stream: torch.cuda.Stream) -> np.ndarray:
        """D2H copy of the interior as float64 in the user's shape."""
        with torch.cuda.stream(stream):
            host = torch.empty(self.kshape, dtype=self.dtype, pin_memory=True)
            host.copy_(self.view(src), non_blocking=True)
        stream.synchronize()
        return host.numpy().astype(np.float64).reshape(self.user_shape)


def boundary_struct(sim, grid: DeviceGrid, nfields: int) -> L.PpfBoundary:
    """PpfBoundary from the simulation's boundary types and the per-face
    constants of _boundary_conditions_array (field j, axis a, side s). A face
    whose values are not uniform is rejected: the library takes one constant
    per face."""
    nd = len(grid.user_shape)
    bcs = bc_per_axis(sim, nd)
    off = len(grid.kshape) - nd
    b = L.PpfBoundary()
    b.reserved = 0
    if off:
        b.type[0] = L.PPF_BC_PERIODIC
    arr = sim._boundary_conditions_array
    for a, name in enumerate(bcs):
        b.type[a + off] = BC_CODES[name]
        if arr is None or name == "PERIODIC":
            continue
        for j in range(min(nfields, 2)):
            for side, k in ((0, 0), (1, -1)):
                idx = tuple(k if ax == a else slice(1, -1) for ax in range(nd))
                face = np.asarray(arr[j][idx], dtype=np.float64)
                v = float(face.flat[0]) if face.size else 0.0
                if face.size and not np.all(face == v):
                    raise NotImplementedError(
                        f"field {j}: non-uniform boundary values on axis {a} side {side}; "
                        "the GB300 engines take one constant per face")
                b.value[j][a + off][side] = v
    return b


def tiling_struct(depth=1, tile=None, pdl=True, flags=0, zchunk=0) -> L.PpfTiling:
    t = L.PpfTiling()
    t.depth = int(depth)
    t.tile_x, t.tile_y = (int(tile[0]), int(tile[1])) if tile else (0, 0)
    t.pdl = 1 if pdl else 0
    t.flags = int(flags)
    t.zchunk = int(zchunk or 0)
    return t


def ptr(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)
