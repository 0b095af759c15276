"""ctypes binding of libcmpy_ed.so (the C ABI declared in include/cmpy_ed.h).

The library is the only compute path: if it is missing this module raises instead of
falling back to anything on the CPU. Device buffers are passed as raw pointers taken from
torch CUDA tensors; streams are torch's current CUDA stream.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "libcmpy_ed.so"
_lock = threading.Lock()
_lib = None

ED_OK = 0
ED_ERR_INVALID_ARG = 1
ED_ERR_CUDA = 2
ED_ERR_TIMEOUT = 3
ED_ERR_NONFINITE = 4
ED_ERR_TOO_LARGE = 5
ED_ERR_ZERO_VECTOR = 6
ED_ERR_DEVICE = 7
ED_ERR_NOT_FOUND = 8


class EDError(RuntimeError):
    """An ed_status != ED_OK returned by the native library."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class FermionModel(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int32),
        ("n_bonds", C.c_int32),
        ("sign_width", C.c_int32),
        ("reserved", C.c_int32),
        ("h_eps", C.POINTER(C.c_double)),
        ("h_u", C.POINTER(C.c_double)),
        ("h_bond_site1", C.POINTER(C.c_int32)),
        ("h_bond_site2", C.POINTER(C.c_int32)),
        ("h_bond_hop", C.POINTER(C.c_double)),
    ]


class SpinModel(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int32),
        ("n_pairs", C.c_int32),
        ("h_pos1", C.POINTER(C.c_int32)),
        ("h_pos2", C.POINTER(C.c_int32)),
        ("h_j", C.POINTER(C.c_double)),
        ("h_jz", C.POINTER(C.c_double)),
    ]


class PlanInfo(C.Structure):
    _fields_ = [
        ("dim", C.c_int64),
        ("num_up", C.c_int64),
        ("num_dn", C.c_int64),
        ("hop_up", C.c_int64),
        ("hop_dn", C.c_int64),
        ("nnz", C.c_int64),
        ("n_sites", C.c_int32),
        ("kind", C.c_int32),
        ("n_up", C.c_int32),
        ("n_dn", C.c_int32),
        ("hnorm_bound", C.c_double),
    ]


class LanczosParams(C.Structure):
    _fields_ = [
        ("max_steps", C.c_int32),
        ("reorth", C.c_int32),
        ("check_every", C.c_int32),
        ("want_vector", C.c_int32),
        ("tol", C.c_double),
        ("seed", C.c_uint64),
        ("profile", C.c_int32),
        ("arithmetic", C.c_int32),
    ]


class LanczosResult(C.Structure):
    _fields_ = [
        ("energy", C.c_double),
        ("residual", C.c_double),
        ("matvec_ms", C.c_double),
        ("steps", C.c_int32),
        ("converged", C.c_int32),
        ("status", C.c_int32),
        ("matvecs", C.c_int32),
    ]


P = C.c_void_p
I32 = C.c_int
I64 = C.c_int64
F64 = C.c_double
PLAN = C.c_void_p

# name: (restype, argtypes)
_SIGNATURES = {
    "ed_status_string": (C.c_char_p, [I32]),
    "ed_last_error": (C.c_char_p, []),
    "ed_version": (I32, []),
    "ed_launch_count": (C.c_uint64, []),
    "ed_binomial": (I64, [I32, I32]),
    "ed_sector_size": (I64, [I32, I32]),
    "ed_enumerate": (I32, [I32, I32, P, I64, P]),
    "ed_rank": (I32, [P, I64, P, P]),
    "ed_plan_create_fermion": (I32, [C.POINTER(FermionModel), I32, I32, C.POINTER(PLAN), P]),
    "ed_plan_create_spin": (I32, [C.POINTER(SpinModel), I32, C.POINTER(PLAN), P]),
    "ed_plan_destroy": (I32, [PLAN]),
    "ed_plan_get_info": (I32, [PLAN, C.POINTER(PlanInfo)]),
    "ed_plan_states": (I32, [PLAN, C.POINTER(P), C.POINTER(P)]),
    "ed_matvec": (I32, [PLAN, P, P, P]),
    "ed_matmat": (I32, [PLAN, P, P, I64, I64, P]),
    "ed_dense": (I32, [PLAN, P, P]),
    "ed_diagonal": (I32, [PLAN, P, P]),
    "ed_csr_matvec": (I32, [I64, P, P, P, P, P, P]),
    "ed_coo_onsite": (I32, [P, I64, P, I64, C.POINTER(F64), I32, P, P, P, I64, C.POINTER(I64), P]),
    "ed_coo_inter": (I32, [P, I64, P, I64, C.POINTER(F64), I32, P, P, P, I64, C.POINTER(I64), P]),
    "ed_coo_hopping": (I32, [P, I64, P, I64, I32, I32, I32, F64, P, P, P, I64, C.POINTER(I64), P]),
    "ed_coo_plan": (I32, [PLAN, P, P, P, I64, C.POINTER(I64), P]),
    "ed_apply_fermion": (I32, [PLAN, PLAN, I32, I32, I32, I32, P, P, I64, I64, I64, P]),
    "ed_apply_fermion_batch": (I32, [P, P, I32, I32, I32, I32, I32, P, P, P, P, P]),
    "ed_lanczos_workspace": (I32, [PLAN, C.POINTER(LanczosParams), C.POINTER(C.c_size_t)]),
    "ed_lanczos": (
        I32,
        [PLAN, C.POINTER(LanczosParams), P, P, C.c_size_t, P, P, P, C.POINTER(LanczosResult), P],
    ),
    "ed_lanczos_coeffs": (I32, [PLAN, I32, P, P, C.c_size_t, P, P, C.POINTER(I32), C.POINTER(F64), P]),
    "ed_lanczos_coeffs_multi": (I32, [I32, P, I32, P, P, P, P, P, P, P, P]),
    "ed_tridiag_lowest": (I32, [P, P, I32, P, P, P]),
    "ed_tridiag_lowest_noalloc": (I32, [P, P, I32, P, P, P]),
    "ed_tridiag_lowest_batch": (I32, [P, I32, P, I32, P, I32, I32, P, P, I32, P]),
    "ed_tridiag_pinv_solve_batch": (I32, [P, I32, P, I32, P, I32, I32, P, P, I32, P, P, I32, P]),
    "ed_dense_eigh_batch": (I32, [P, I64, I64, P, I32, I32, P, P, I64, I64, P]),
    "ed_tridiag_eigh": (I32, [P, P, I32, P, P, I64, P]),
    "ed_batch_create": (I32, [C.POINTER(C.c_void_p), I32, C.POINTER(C.c_void_p)]),
    "ed_batch_destroy": (I32, [C.c_void_p]),
    "ed_batch_workspace": (I32, [C.c_void_p, I32, I32, I32, I32, C.POINTER(C.c_size_t)]),
    "ed_batch_lanczos": (
        I32,
        [C.c_void_p, I32, F64, I32, C.c_uint64, P, I32, P, C.c_size_t, P, P, P, P, P, P, P, I32, I32, I32, P],
    ),
    "ed_batch_tune": (
        I32,
        [C.c_void_p, I32, P, C.c_size_t, P, P, P, P, P, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32),
         C.POINTER(C.c_float), P],
    ),
    "ed_batch_gf_continued_fraction": (I32, [I32, I32, P, P, P, P, I32, P, I64, P, P]),
    "ed_plan_num_params": (I32, [PLAN]),
    "ed_param_sandwich": (I32, [PLAN, P, P, P, I32, P]),
    "ed_tape_workspace": (I32, [PLAN, I32, I32, C.POINTER(C.c_size_t)]),
    "ed_lanczos_tape": (I32, [PLAN, P, I32, I32, F64, I32, F64, P, C.c_size_t, P, P, P, C.POINTER(C.c_int), P]),
    "ed_tape_combine": (I32, [PLAN, I32, I32, P, P, P, P, P, P, P, P, C.c_size_t, P]),
    "ed_tape_reverse": (I32, [PLAN, I32, I32, P, P, P, P, P, P, P, P, C.c_size_t, P, P, P]),
    "ed_cf_adjoint": (I32, [P, P, I32, F64, F64, I32, P, I64, P, P, P, P, P]),
    "ed_batch_diag": (I32, [PLAN, I32, P, P, P]),
    "ed_batch_cf": (I32, [I32, P, I64, P, I64, P, P, P, I32, P, I64, P, P]),
    "ed_batch_cf_adjoint": (I32, [I32, P, I64, P, I64, P, I32, P, P, I32, P, I64, P, P, P, P, P]),
    "ed_batch_matvec_params": (I32, [PLAN, I32, P, P, P, P, P]),
    "ed_batch_tape_workspace": (I32, [PLAN, I32, I32, I32, C.POINTER(C.c_size_t)]),
    "ed_batch_lanczos_tape": (I32, [PLAN, I32, P, P, P, I32, I32, F64, I32, F64, P, C.c_size_t, P, P, P,
                                    C.POINTER(C.c_int), P]),
    "ed_batch_tape_combine": (I32, [PLAN, I32, P, P, C.POINTER(C.c_int), I32, I32, P, P, P, P, P, P, P, P,
                                    C.c_size_t, P]),
    "ed_batch_tape_reverse": (I32, [PLAN, I32, P, P, C.POINTER(C.c_int), I32, I32, P, P, P, P, P, P, P, P,
                                    C.c_size_t, P, P, P]),
    "ed_plan_fixed_point": (I32, [PLAN]),
    "ed_fixed_from_f64": (I32, [P, I64, I32, P, C.POINTER(C.c_int32), P]),
    "ed_fixed_to_f64": (I32, [P, I64, C.c_int32, P, P]),
    "ed_matvec_fixed": (I32, [PLAN, P, C.c_int32, P, C.POINTER(C.c_int32), C.POINTER(I32), P]),
    "ed_plan_matvec_variant": (I32, [PLAN]),
    "ed_plan_set_wait_limit": (I32, [PLAN, I64]),
    "ed_plan_set_matvec_variant": (I32, [PLAN, I32]),
    "ed_gf_continued_fraction": (I32, [P, P, I32, F64, F64, I32, P, I64, P, I32, P]),
    "ed_lehmann_accumulate": (I32, [P, I64, P, I64, P, F64, F64, P, I64, P, P]),
    "ed_tevo_sum": (I32, [P, P, I64, F64, I32, P, I64, P, I32, P]),
    "ed_laplace_t2z": (I32, [P, P, I64, P, I64, I32, P, P]),
}


def library_path() -> Path:
    return _LIB_PATH


def lib():
    """The loaded libcmpy_ed.so (loaded once). Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not _LIB_PATH.exists():
                raise RuntimeError(
                    f"{_LIB_PATH.name} is not built: run `python -m cmpy_gb300.build` "
                    "(needs the CUDA toolkit); there is no CPU fallback"
                )
            h = C.CDLL(str(_LIB_PATH))
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(h, name)
                fn.restype = res
                fn.argtypes = args
            _lib = h
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def check(status: int) -> None:
    if status != ED_OK:
        L = lib()
        msg = L.ed_last_error().decode(errors="replace")
        if status == ED_ERR_INVALID_ARG:
            raise ValueError(f"{msg} [ed_status {status}]")
        raise EDError(status, msg)


def ptr(t) -> int | None:
    """Raw device pointer of a torch CUDA tensor (None for None)."""
    if t is None:
        return None
    return t.data_ptr()


def stream_handle(stream=None) -> int | None:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def f64_array(values) -> tuple[np.ndarray, C.POINTER(C.c_double)]:
    a = np.ascontiguousarray(values, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def i32_array(values) -> tuple[np.ndarray, C.POINTER(C.c_int32)]:
    a = np.ascontiguousarray(values, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int32))
