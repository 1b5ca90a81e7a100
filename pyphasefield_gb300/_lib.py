"""ctypes binding of libppf_gb300.so (declared in include/ppf_gb300.h).

The library is the only compute path: if it cannot be loaded, every engine
call raises. Nothing here falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libppf_gb300.so"

PPF_ABI_VERSION = 3  # the struct layouts and signatures below
PPF_OK = 0
PPF_ERR_INVALID = -1
PPF_ERR_CUDA = -2
PPF_ERR_UNSUPPORTED = -3
PPF_ERR_TIMEOUT = -4
PPF_ERR_NONFINITE = -5

PPF_BC_PERIODIC = 0
PPF_BC_NEUMANN = 1
PPF_BC_DIRCHLET = 2

PPF_STATUS_NONFINITE = 1
PPF_STATUS_TIMEOUT = 2
PPF_STATUS_RANGE = 4
PPF_STATUS_NOT_CONVERGED = 8


class PpfError(RuntimeError):
    """A libppf_gb300 call returned a negative status."""

    def __init__(self, code: int, func: str, msg: str):
        super().__init__(f"{func} failed with status {code}: {msg}")
        self.code = code


class PpfGrid(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("reserved", C.c_int32),
                ("shape", C.c_int64 * 3), ("pitch", C.c_int64)]


class PpfBoundary(C.Structure):
    _fields_ = [("type", C.c_int32 * 3), ("reserved", C.c_int32),
                ("value", ((C.c_double * 2) * 3) * 2)]


class PpfTiling(C.Structure):
    _fields_ = [("depth", C.c_int32), ("tile_x", C.c_int32), ("tile_y", C.c_int32),
                ("pdl", C.c_int32), ("flags", C.c_int32), ("zchunk", C.c_int32)]


PPF_TILING_FULL_EVAL = 1


class PpfDiffusionParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dx", "dt", "D")]


class PpfAllenCahnParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dx", "dt", "M", "epsilon", "W")]


class PpfCahnHilliardParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dx", "dt", "M", "epsilon", "quantum")] + [
        ("centered", C.c_int32), ("reserved", C.c_int32)]


WARREN_PARAM_NAMES = ("dx", "dt", "T_mA", "T_mB", "L_A", "L_B", "D_L", "D_S", "v_m",
                      "R", "y_e", "T", "alpha", "ebar", "W_A", "W_B", "M_A", "M_B")


class PpfWarren1995Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in WARREN_PARAM_NAMES]


PPF_SOLVER_EXPLICIT = 0
PPF_SOLVER_IMPLICIT = 1
PPF_SOLVER_CRANK_NICOLSON = 2
PPF_SOLVER_IMEX = 3
PPF_MODEL_CAHN_HILLIARD = 3


class PpfImplicitPhaseParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dx", "dt", "M", "W", "epsilon", "tol")] + [
        (n, C.c_int32) for n in ("model", "solver", "adi", "gmres", "max_iter", "reserved")]


class PpfImplicitDiffusionParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dx", "dt", "D", "tol")] + [
        ("solver", C.c_int32), ("adi", C.c_int32)]


PPF_NCGPU_MAX_COMP = 6
PPF_NCGPU_MAX_EXCESS = 16
PPF_NCGPU_VARIANT_NCGPU = 0
PPF_NCGPU_VARIANT_NEW = 1


class PpfNcgpuExcess(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("phase", "a", "b", "order", "npieces", "reserved")] + [
        ("piece", (C.c_double * 10) * 4)]


class PpfNcgpuParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dx", "dt", "v_m", "D_L", "D_S", "M_qmax", "H",
                                          "y_e", "beta", "ebar2", "noise_scale")] + [
        ("W", C.c_double * PPF_NCGPU_MAX_COMP), ("M", C.c_double * PPF_NCGPU_MAX_COMP),
        ("gibbs", (((C.c_double * 10) * 4) * PPF_NCGPU_MAX_COMP) * 2),
        ("npieces", (C.c_int32 * PPF_NCGPU_MAX_COMP) * 2),
        ("ncomp", C.c_int32), ("nexcess", C.c_int32),
        ("excess", PpfNcgpuExcess * PPF_NCGPU_MAX_EXCESS),
        ("variant", C.c_int32), ("reserved", C.c_int32),
        ("eqbar2", C.c_double), ("noise_phi", C.c_double), ("noise_q", C.c_double)]


PPF_MODEL_WARREN1995 = 1
PPF_MODEL_ALLEN_CAHN = 2


class PpfMember(C.Structure):
    _fields_ = [("model", C.c_int32), ("reserved", C.c_int32), ("ny", C.c_int64),
                ("nx", C.c_int64), ("pitch", C.c_int64), ("bc", PpfBoundary),
                ("phi", C.c_void_p * 2), ("c", C.c_void_p * 2), ("seed", C.c_uint64),
                ("w95", PpfWarren1995Params), ("ac", PpfAllenCahnParams)]


class PpfEnsemblePlan(C.Structure):
    _fields_ = [("device_table", C.c_void_p), ("n_items", C.c_int64),
                ("n_members", C.c_int32), ("rows", C.c_int32), ("n_units", C.c_int64),
                ("bands", C.c_int32), ("reserved", C.c_int32)]


class PpfSgShape(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("B", "H", "W", "pitch", "P", "C", "E")] + [
        (n, C.c_float) for n in ("s0", "s1", "in_off0", "in_sc0", "in_off1", "in_sc1",
                                 "lo0", "hi0", "lo1", "hi1")]


P = C.c_void_p
I32 = C.c_int32
U64 = C.c_uint64
SZ = C.c_size_t
PG, PB, PT = C.POINTER(PpfGrid), C.POINTER(PpfBoundary), C.POINTER(PpfTiling)

# name -> argtypes; every function returns int32 status.
SIGNATURES: dict[str, list] = {
    "ppf_version": [C.POINTER(I32), C.c_char_p, SZ],
    "ppf_last_error": [C.c_char_p, SZ],
    "ppf_device_info": [I32, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)],
    "ppf_diffusion_step_f32": [C.POINTER(PpfDiffusionParams), PG, PB, P, P, PT, P],
    "ppf_diffusion_step_f64": [C.POINTER(PpfDiffusionParams), PG, PB, P, P, PT, P],
    "ppf_allen_cahn_step_f32": [C.POINTER(PpfAllenCahnParams), PG, PB, P, P, PT, P],
    "ppf_allen_cahn_step_f64": [C.POINTER(PpfAllenCahnParams), PG, PB, P, P, PT, P],
    "ppf_cahn_hilliard_step_f32": [C.POINTER(PpfCahnHilliardParams), PG, PB, P, P, P, P, PT, P],
    "ppf_cahn_hilliard_step_f64": [C.POINTER(PpfCahnHilliardParams), PG, PB, P, P, P, P, PT, P],
    "ppf_warren1995_step_f32": [C.POINTER(PpfWarren1995Params), PG, PB, P, P, P, P, U64, U64, P, PT, P],
    "ppf_warren1995_step_f64": [C.POINTER(PpfWarren1995Params), PG, PB, P, P, P, P, U64, U64, P, PT, P],
    "ppf_implicit_scratch_bytes": [PG, I32, C.POINTER(SZ)],
    "ppf_diffusion_implicit_step_f32": [C.POINTER(PpfImplicitDiffusionParams), PG, P, P, P, P,
                                        SZ, C.POINTER(I32), P],
    "ppf_diffusion_implicit_step_f64": [C.POINTER(PpfImplicitDiffusionParams), PG, P, P, P, P,
                                        SZ, C.POINTER(I32), P],
    "ppf_ncgpu_step_f32": [C.POINTER(PpfNcgpuParams), PG, PB, P, P, P, P, P, U64, U64, P, P],
    "ppf_ncgpu_step_f64": [C.POINTER(PpfNcgpuParams), PG, PB, P, P, P, P, P, U64, U64, P, P],
    "ppf_ncgpu_tables_f32": [C.POINTER(PpfNcgpuParams), PG, P, P, P],
    "ppf_ncgpu_tables_f64": [C.POINTER(PpfNcgpuParams), PG, P, P, P],
    "ppf_ncgpu_temperature_advance_f32": [PG, P, C.c_double, P],
    "ppf_ncgpu_temperature_advance_f64": [PG, P, C.c_double, P],
    "ppf_phase_implicit_scratch_bytes": [PG, I32, C.POINTER(SZ)],
    "ppf_phase_implicit_step_f32": [C.POINTER(PpfImplicitPhaseParams), PG, P, P, P, P, SZ,
                                    C.POINTER(I32), P],
    "ppf_phase_implicit_step_f64": [C.POINTER(PpfImplicitPhaseParams), PG, P, P, P, P, SZ,
                                    C.POINTER(I32), P],
    "ppf_var_line_solve_f32": [PG, I32, C.c_double, C.c_double, C.c_double, P, I32, C.c_double,
                               P, P, P, SZ, P],
    "ppf_var_line_solve_f64": [PG, I32, C.c_double, C.c_double, C.c_double, P, I32, C.c_double,
                               P, P, P, SZ, P],
    "ppf_line_solve_f32": [PG, I32, C.c_double, I32, C.c_double, P, P, P, SZ, P],
    "ppf_line_solve_f64": [PG, I32, C.c_double, I32, C.c_double, P, P, P, SZ, P],
    "ppf_periodic_solve_f32": [PG, C.c_double, C.c_double, C.c_double, P, P, P,
                               C.POINTER(I32), P],
    "ppf_periodic_solve_f64": [PG, C.c_double, C.c_double, C.c_double, P, P, P,
                               C.POINTER(I32), P],
    "ppf_ensemble_plan_bytes": [C.POINTER(PpfMember), I32, PT, C.POINTER(SZ)],
    "ppf_ensemble_build": [C.POINTER(PpfMember), I32, PT, P, SZ, C.POINTER(PpfEnsemblePlan), P],
    "ppf_ensemble_step_f32": [C.POINTER(PpfEnsemblePlan), I32, U64, P, PT, P],
    "ppf_ensemble_run_f32": [C.POINTER(PpfEnsemblePlan), I32, U64, P, I32, P, PT, P],
    "ppf_sg_gemm": [P, C.c_longlong, C.c_longlong, P, C.c_longlong, C.c_longlong, P,
                    C.c_longlong, P, I32, C.c_longlong, C.c_longlong, C.c_longlong, I32, P],
    "ppf_sg_patch_fwd": [C.POINTER(PpfSgShape), P, P, P, P, P, P],
    "ppf_sg_patch_bwd_weight": [C.POINTER(PpfSgShape), P, P, P, P, P],
    "ppf_sg_residual": [C.POINTER(PpfSgShape), P, P, P, C.c_int32, P, P],
    "ppf_sg_block_fwd": [C.POINTER(PpfSgShape)] + [P] * 14,
    "ppf_sg_block_bwd": [C.POINTER(PpfSgShape)] + [P] * 20,
    "ppf_sg_head_fwd": [C.POINTER(PpfSgShape), P, P, P, P, P],
    "ppf_sg_head_bwd": [C.POINTER(PpfSgShape), P, P, P, P, P, P, P, P],
    "ppf_sg_mse": [C.POINTER(PpfSgShape), P, P, P, P, P, P],
    "ppf_sg_apply": [C.POINTER(PpfSgShape), P, P, P, P],
    "ppf_sg_cast_bf16": [P, P, C.c_longlong, P],
    "ppf_sg_set_tensor_path": [C.c_int32],
    "ppf_sg_adam": [P, P, P, P, P, C.c_longlong, C.c_float, C.c_float, C.c_float, C.c_float,
                    I32, C.c_float, P],
    "ppf_reduce_scratch_bytes": [PG, C.POINTER(SZ)],
    "ppf_reduce_sum_f32": [P, PG, P, P, SZ, P],
    "ppf_reduce_sum_f64": [P, PG, P, P, SZ, P],
    "ppf_reduce_sum_f32_noalloc": [P, PG, P, P],
    "ppf_free_energy_f32": [P, PG, PB, C.c_double, C.c_double, C.c_double, P, P, SZ, P],
    "ppf_free_energy_f64": [P, PG, PB, C.c_double, C.c_double, C.c_double, P, P, SZ, P],
    "ppf_check_finite_f32": [P, PG, P, P],
    "ppf_check_finite_f64": [P, PG, P, P],
    "ppf_status_take": [C.POINTER(I32)],
    "ppf_status_collect": [P, P],
    "ppf_selftest_wait_timeout": [I32, P],
    "ppf_counter_add_u64": [P, U64, P],
    "ppf_graph_begin": [P],
    "ppf_graph_end": [P, C.POINTER(P)],
    "ppf_graph_launch": [P, P],
    "ppf_graph_destroy": [P],
}

_lib = None
_lock = threading.Lock()


def load(path: str | Path | None = None):
    """Load the shared library once (raises OSError if it is missing)."""
    global _lib
    with _lock:
        if _lib is None:
            p = Path(path) if path else LIB_PATH
            if not p.exists():
                raise OSError(
                    f"{p} not found: build it with `python -m pyphasefield_gb300.build` "
                    "(the CUDA library is the only compute path)")
            lib = C.CDLL(str(p))
            # the ABI first: a library of another ABI may lack symbols bound below
            lib.ppf_version.argtypes = [C.POINTER(I32), C.c_char_p, SZ]
            lib.ppf_version.restype = C.c_int32
            abi = I32()
            buf = C.create_string_buffer(128)
            lib.ppf_version(C.byref(abi), buf, len(buf))
            if abi.value != PPF_ABI_VERSION:
                raise OSError(f"{p} has ABI {abi.value}, this binding {PPF_ABI_VERSION}: "
                              "rebuild it with `python -m pyphasefield_gb300.build`")
            for name, argtypes in SIGNATURES.items():
                try:
                    fn = getattr(lib, name)
                except AttributeError:
                    raise OSError(f"{p} lacks {name}: rebuild it with "
                                  "`python -m pyphasefield_gb300.build`") from None
                fn.argtypes = argtypes
                fn.restype = C.c_int32
            _lib = lib
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(512)
    load().ppf_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def call(name: str, *args) -> None:
    """Call a library function and raise PpfError on a negative status."""
    rc = getattr(load(), name)(*args)
    if rc != PPF_OK:
        raise PpfError(rc, name, last_error())


def version() -> tuple[int, str]:
    abi = I32()
    buf = C.create_string_buffer(128)
    call("ppf_version", C.byref(abi), buf, len(buf))
    return abi.value, buf.value.decode()
