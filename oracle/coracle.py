"""ctypes front end of the C restatement of the Warren1995 step
(oracle/warren_c.c).

TEST INFRASTRUCTURE ONLY: the GPU parity tests use it as the checker on grids
where the numpy restatement (oracle/restate.py) would take minutes, and
tests/test_oracle.py pins it to that numpy restatement. Nothing in the
shipped package imports it.

build() compiles oracle/libppf_oracle.so with gcc (-O2, -ffp-contract=off so
that no multiply-add is fused and every operation rounds as numpy's does;
OpenMP when the compiler has it). run_warren() has the signature and
meaning of oracle.restate.run_warren.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "warren_c.c"
LIB = HERE / "libppf_oracle.so"
_BC = {"PERIODIC": 0, "NEUMANN": 1, "DIRCHLET": 2}
_lib = None


class _Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "W_A", "W_B", "L_A", "L_B", "T", "T_mA", "T_mB", "D_S", "D_L", "v_m", "R", "y_e",
        "M_A", "M_B", "ebar", "alpha", "ebar2")]


def _stamp() -> str:
    h = hashlib.sha256(SRC.read_bytes())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False) -> Path:
    """Compile the oracle library (seconds); skipped when up to date."""
    stamp = HERE / ".libppf_oracle.stamp"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == _stamp():
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle library")
    base = [cc, "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            str(SRC), "-o", str(LIB) + ".tmp", "-lm"]
    r = subprocess.run(base[:2] + ["-fopenmp"] + base[2:], capture_output=True, text=True)
    if r.returncode != 0:  # no OpenMP: single-threaded
        r = subprocess.run(base, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(str(LIB) + ".tmp", LIB)
    stamp.write_text(_stamp())
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.ppf_oracle_warren_run.restype = C.c_int
        L.ppf_oracle_warren_run.argtypes = [
            C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(_Params), C.c_double,
            C.c_double, C.POINTER(C.c_int), C.c_void_p, C.c_uint64, C.c_uint64, C.c_int]
        _lib = L
    return _lib


def run_warren(phi0: np.ndarray, c0: np.ndarray, steps: int, boundary_conditions,
               dx: float, params: dict, seed: int = 0, step0: int = 0,
               values=None) -> tuple[np.ndarray, np.ndarray]:
    """oracle.restate.run_warren in C: same arguments, same results up to the
    last bits of the C library's atan2/cos/sin."""
    from .restate import bc_list, fill_ghosts, interior, pad, warren_derived

    p = warren_derived(params, dx)
    phi = pad(np.asarray(phi0, dtype=np.float64))
    c = pad(np.asarray(c0, dtype=np.float64))
    bcs = bc_list(boundary_conditions, 2)
    fill_ghosts([phi, c], bcs, dx, values)
    phi = np.ascontiguousarray(phi)
    c = np.ascontiguousarray(c)
    prm = _Params(**{k: float(p[k]) for k, _ in _Params._fields_ if k != "ebar2"},
                  ebar2=float(p["ebar"] ** 2))
    bc = (C.c_int * 2)(*(_BC[b] for b in bcs))
    vals = None
    if values is not None:
        v = np.zeros((2, 2, 2))
        for j in range(min(2, len(values))):
            v[j] = np.asarray(values[j], dtype=np.float64)
        vals = np.ascontiguousarray(v)
    rc = lib().ppf_oracle_warren_run(
        phi.ctypes.data, c.ctypes.data, phi0.shape[0], phi0.shape[1], C.byref(prm), float(dx),
        float(p["dt"]), bc, vals.ctypes.data if vals is not None else None, int(seed),
        int(step0), int(steps))
    if rc != 0:
        raise MemoryError("oracle: out of host memory")
    return interior(phi).copy(), interior(c).copy()
