"""ctypes binding of ``liboqupy_gb300.so`` (declared in include/oqupy_gb300.h).

The library is the only compute path of this package: if it cannot be
loaded, every entry point raises.  There is no CPU fallback.
"""

import ctypes
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboqupy_gb300.so")

OTB_OK = 0
# largest bond split (columns) one CTA handles: chi_cap * D <= MAX_COLUMNS
MAX_COLUMNS = 1152

OTB_ERR_INVALID_ARG = -1
OTB_ERR_OOM = -2
OTB_ERR_CUDA = -3
OTB_ERR_NO_CONVERGENCE = -4
OTB_ERR_TIMEOUT = -5
OTB_ERR_NONFINITE = -6
OTB_ERR_CHI_OVERFLOW = -7

PRECISION = {"complex128": 0, "mixed": 1}

STATUS_TEXT = {
    OTB_ERR_INVALID_ARG: "invalid argument",
    OTB_ERR_OOM: "out of device memory",
    OTB_ERR_CUDA: "CUDA error",
    OTB_ERR_NO_CONVERGENCE: "Jacobi SVD did not converge",
    OTB_ERR_TIMEOUT: "device wait timed out",
    OTB_ERR_NONFINITE: "non-finite values in a bond split",
    OTB_ERR_CHI_OVERFLOW: "bond dimension exceeded chi_cap",
}

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int32_p = ctypes.POINTER(ctypes.c_int32)


class TempoConfig(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("chi_cap", ctypes.c_int32),
                ("out_cap", ctypes.c_int32), ("grid", ctypes.c_int32),
                ("block", ctypes.c_int32), ("smem_kb", ctypes.c_int32),
                ("qr_cut", ctypes.c_double)]


class TempoInstance(ctypes.Structure):
    _fields_ = [("hs_dim", ctypes.c_int32), ("dkmax", ctypes.c_int32),
                ("epsrel", ctypes.c_double), ("n_influences", ctypes.c_int32),
                ("influences", c_double_p), ("prop1", c_double_p),
                ("prop2", c_double_p), ("rho0", c_double_p),
                ("max_sites", ctypes.c_int32)]


class TempoInfo(ctypes.Structure):
    _fields_ = [("step", ctypes.c_int32), ("status", ctypes.c_int32),
                ("nsites", ctypes.c_int32), ("max_bond", ctypes.c_int32),
                ("log_scale", ctypes.c_double), ("splits", ctypes.c_int32),
                ("sweeps64", ctypes.c_int32), ("sweeps32", ctypes.c_int32),
                ("flops_alg", ctypes.c_double), ("t_begin_ns", ctypes.c_int64),
                ("t_end_ns", ctypes.c_int64)]


class PtConfig(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("chi_cap", ctypes.c_int32),
                ("grid", ctypes.c_int32), ("qr_cut", ctypes.c_double)]


class PtInstance(ctypes.Structure):
    _fields_ = [("hs_dim", ctypes.c_int32), ("num_steps", ctypes.c_int32),
                ("dkmax", ctypes.c_int32), ("epsrel", ctypes.c_double),
                ("influences", c_double_p), ("neg_influences", c_double_p)]


class PtInfo(ctypes.Structure):
    _fields_ = [("step", ctypes.c_int32), ("status", ctypes.c_int32),
                ("num_steps", ctypes.c_int32), ("max_bond", ctypes.c_int32),
                ("splits", ctypes.c_int32), ("sweeps64", ctypes.c_int32),
                ("sweepsff", ctypes.c_int32), ("caps_done", ctypes.c_int32),
                ("flops_alg", ctypes.c_double)]


class DeviceError(RuntimeError):
    """A status code returned by the CUDA library."""

    def __init__(self, code, msg):
        super().__init__(f"{STATUS_TEXT.get(code, 'error')} ({code}): {msg}")
        self.code = code


_lib: Optional[ctypes.CDLL] = None


def _declare(lib):
    P = ctypes.c_void_p
    i32 = ctypes.c_int32
    sig = {
        "otb_tempo_create": (i32, [ctypes.POINTER(TempoConfig), i32,
                                   ctypes.POINTER(TempoInstance), ctypes.POINTER(P)]),
        "otb_tempo_destroy": (None, [P]),
        "otb_tempo_advance": (i32, [P, i32, P]),
        "otb_tempo_read_states": (i32, [P, i32, i32, i32, c_double_p]),
        "otb_tempo_read_all_states": (i32, [P, i32, i32, c_double_p]),
        "otb_tempo_get_info": (i32, [P, i32, ctypes.POINTER(TempoInfo)]),
        "otb_tempo_bond_dims": (i32, [P, i32, c_int32_p, i32, c_int32_p]),
        "otb_tempo_set_influence": (i32, [P, i32, i32, c_double_p]),
        "otb_tempo_set_propagators": (i32, [P, i32, c_double_p, c_double_p]),
        "otb_tempo_set_all_propagators": (i32, [P, c_double_p, c_double_p, P]),
        "otb_tempo_set_first_influence": (i32, [P, i32, c_double_p]),
        "otb_tempo_reserve_sites": (i32, [P, i32]),
        "otb_tempo_set_launch": (i32, [P, i32, i32, i32]),
        "otb_pt_create": (i32, [ctypes.POINTER(PtConfig), i32,
                                ctypes.POINTER(PtInstance), ctypes.POINTER(P)]),
        "otb_pt_destroy": (None, [P]),
        "otb_pt_advance": (i32, [P, i32, P]),
        "otb_pt_get_info": (i32, [P, i32, ctypes.POINTER(PtInfo)]),
        "otb_pt_bond_dims": (i32, [P, i32, c_int32_p, i32]),
        "otb_pt_get_tensor": (i32, [P, i32, i32, c_double_p, ctypes.c_int64, c_int32_p]),
        "otb_pt_get_cap": (i32, [P, i32, i32, c_double_p, i32, c_int32_p]),
        "otb_dyn_run": (i32, [P, i32, i32, c_double_p, c_double_p, c_double_p, i32,
                              c_double_p, P]),
        "otb_dyn_run_steps": (i32, [P, i32, i32, c_double_p, i32, c_int32_p, c_double_p, i32,
                                    c_double_p, P]),
        "otb_dyn_gradient": (i32, [P, i32, i32, c_double_p, i32, c_int32_p, c_double_p, c_double_p,
                                   i32, c_double_p, c_double_p, P]),
        "otb_dyn_session_create": (i32, [P, i32, i32, c_double_p, ctypes.POINTER(P)]),
        "otb_dyn_session_step": (i32, [P, c_double_p, c_double_p, P]),
        "otb_dyn_session_state": (i32, [P, i32, c_double_p]),
        "otb_dyn_session_destroy": (None, [P]),
        "otb_mlp_gemm": (i32, [P, P, i32, i32, i32, P, i32, P, P, P, P, P, P]),
        "otb_mlp_transpose_bf16": (i32, [P, P, i32, i32, P]),
        "otb_mlp_f32_to_bf16": (i32, [P, P, ctypes.c_int64, P]),
        "otb_mlp_colsum": (i32, [P, P, i32, i32, P]),
        "otb_mlp_bloch_free_add": (i32, [P, P, i32, i32, ctypes.c_float, P]),
        "otb_mlp_mse_grad": (i32, [P, P, P, P, ctypes.c_int64, P, P]),
        "otb_mlp_adamw": (i32, [P, P, P, P, P, ctypes.c_int64, ctypes.c_float,
                                ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                ctypes.c_float, i32, P]),
        "otb_measure_fma_peak": (i32, [i32, c_double_p]),
        "otb_last_error": (ctypes.c_char_p, []),
        "otb_version": (i32, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return sig


def exported_symbols():
    """Names the header declares and this binding calls."""
    return [
        "otb_tempo_create", "otb_tempo_destroy", "otb_tempo_advance",
        "otb_tempo_read_states", "otb_tempo_read_all_states",
        "otb_tempo_get_info", "otb_tempo_bond_dims", "otb_tempo_set_influence",
        "otb_tempo_set_propagators", "otb_tempo_set_all_propagators", "otb_tempo_set_first_influence",
        "otb_tempo_reserve_sites", "otb_tempo_set_launch", "otb_pt_create", "otb_pt_destroy",
        "otb_pt_advance", "otb_pt_get_info", "otb_pt_bond_dims",
        "otb_pt_get_tensor", "otb_pt_get_cap", "otb_dyn_run", "otb_dyn_run_steps", "otb_dyn_gradient", "otb_dyn_session_create",
        "otb_dyn_session_step", "otb_dyn_session_state", "otb_dyn_session_destroy", "otb_mlp_gemm",
        "otb_mlp_transpose_bf16", "otb_mlp_f32_to_bf16", "otb_mlp_colsum",
        "otb_mlp_mse_grad", "otb_mlp_adamw", "otb_mlp_bloch_free_add",
        "otb_measure_fma_peak", "otb_last_error", "otb_version"]


def fma_peak_tflops(precision: int) -> float:
    """Measured FMA-pipe peak of the current GPU (0 = FP64, 1 = FP32)."""
    v = ctypes.c_double()
    check(lib().otb_measure_fma_peak(int(precision), ctypes.byref(v)))
    return v.value


def lib() -> ctypes.CDLL:
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: run oqupy_gb300.build.build() first "
                "(the GPU path has no CPU fallback)")
        l = ctypes.CDLL(LIB_PATH)
        _declare(l)
        _lib = l
    return _lib


def check(code: int):
    if code != OTB_OK:
        msg = lib().otb_last_error().decode(errors="replace")
        raise DeviceError(code, msg)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(c_double_p)


def cplx(a) -> np.ndarray:
    """complex array -> contiguous interleaved float64 view."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    return a.view(np.float64).reshape(a.shape + (2,))
