"""ctypes binding of ``libfdtd_gb300.so`` (declarations in ``include/fdtd.h``).

The library is the only compute path: if it is missing or cannot be loaded,
every call raises ``FdtdLibraryError``; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

FDTD_OK = 0
ERR = {
    -1: "FDTD_ERR_NULL", -2: "FDTD_ERR_SIZE", -3: "FDTD_ERR_ALIGN", -4: "FDTD_ERR_ARG",
    -5: "FDTD_ERR_CUDA", -6: "FDTD_ERR_NONFINITE", -7: "FDTD_ERR_TIMEOUT",
    -8: "FDTD_ERR_UNSUPPORTED", -9: "FDTD_ERR_WORKSPACE",
}
SRC_NONE, SRC_HARD, SRC_SOFT = 0, 1, 2
FORM_CB, FORM_CACB, FORM_DFORM, FORM_DEBYE = 0, 1, 2, 3
MAX_PROBES = 8
STATUS_NONFINITE, STATUS_TIMEOUT, STATUS_BOUNDS = 1, 2, 4


class FdtdLibraryError(RuntimeError):
    pass


class FdtdError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        name = ERR.get(code, str(code))
        msg = f"{where}: {name}"
        try:
            msg += f" ({lib().fdtd_status_string(code).decode()})"
            if code == -5:
                msg += f", cudaError {lib().fdtd_last_cuda_error()}"
        except Exception:  # pragma: no cover
            pass
        super().__init__(msg)


P = C.c_void_p
F = C.c_void_p  # float* (device)


class Pml2D(C.Structure):
    _fields_ = [(n, F) for n in ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3", "gx2", "gx3", "gy2", "gy3")]


class Source2D(C.Structure):
    _fields_ = [("kind", C.c_int), ("i", C.c_int), ("j", C.c_int), ("table", F), ("table_len", C.c_int)]


class Params2D(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("pml", Pml2D), ("naz", F), ("nbz", F), ("src", Source2D),
                ("tfsf_npml", C.c_int), ("tfsf_table", F), ("tfsf_table_len", C.c_int),
                ("nf", C.c_int), ("dft_cos", F), ("dft_sin", F), ("dft_table_len", C.c_int),
                ("probe_i", C.c_int), ("probe_j", C.c_int), ("probe_len", C.c_int), ("pml_cells", C.c_int)]


class State2D(C.Structure):
    _fields_ = [(n, F) for n in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy", "ezi", "hxi", "bc",
                                 "r_pt", "i_pt", "r_in", "i_in")] + [("status", P), ("probe_ez", F)]


class Fields2D(C.Structure):
    _fields_ = [(n, F) for n in ("dz", "iz", "hx", "hy", "ihx", "ihy")]


class Box2D(C.Structure):
    _fields_ = [("i0", C.c_int), ("j0", C.c_int), ("ni", C.c_int), ("nj", C.c_int)]


class AdjointParams2D(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("checkpoint", C.c_int), ("probe_i", C.c_int), ("probe_j", C.c_int),
                ("probe_weight", C.c_float), ("box", Box2D)]


class GemmDesc(C.Structure):
    _fields_ = [("M", C.c_int), ("N", C.c_int), ("K", C.c_int), ("batch", C.c_int),
                ("A", P), ("lda", C.c_longlong), ("stride_a", C.c_longlong), ("a_mn_major", C.c_int),
                ("B", P), ("ldb", C.c_longlong), ("stride_b", C.c_longlong), ("b_mn_major", C.c_int),
                ("C32", P), ("C16", P), ("ldc", C.c_longlong), ("stride_c", C.c_longlong),
                ("bias", P), ("res16", P), ("ldr", C.c_longlong), ("stride_r", C.c_longlong),
                ("alpha", C.c_float), ("act", C.c_int), ("accumulate", C.c_int), ("pre16", P),
                ("mn_lbo", C.c_int), ("mn_sbo", C.c_int),
                ("K2", C.c_int), ("A2", P), ("lda2", C.c_longlong), ("stride_a2", C.c_longlong), ("a2_mn_major", C.c_int),
                ("B2", P), ("ldb2", C.c_longlong), ("stride_b2", C.c_longlong), ("b2_mn_major", C.c_int)]


class Params1D(C.Structure):
    _fields_ = [("nx", C.c_int), ("form", C.c_int)] + [(n, F) for n in ("ca", "cb", "nax", "nbx", "ncx", "ndx")] + [
        ("src_kind", C.c_int), ("src_k", C.c_int), ("src_table", F), ("src_table_len", C.c_int),
        ("abc", C.c_int), ("nf", C.c_int), ("dft_cos", F), ("dft_sin", F), ("dft_table_len", C.c_int),
        ("nprobe", C.c_int), ("probe_k", C.c_int * MAX_PROBES), ("full_dft", C.c_int)]


class State1D(C.Structure):
    _fields_ = [(n, F) for n in ("ex", "hy", "dx", "ix", "sx", "bc", "r_pt", "i_pt", "r_pr", "i_pr")] + [
        ("status", P)]


class BatchParams1D(C.Structure):
    _fields_ = [("nruns", C.c_int), ("ke", P), ("layer_off", P), ("nlayers", C.c_int), ("layer_start", P),
                ("layer_end", P), ("layer_ca", F), ("layer_cb", F), ("probe_in", P), ("probe_out", P),
                ("src_k", C.c_int), ("src_table", F), ("nsteps", C.c_int), ("nf", C.c_int), ("dft_cos", F),
                ("dft_sin", F)]


class BatchOut1D(C.Structure):
    _fields_ = [("spec", F), ("done", P), ("status", P), ("queue", P)]


_SIGS = {
    "fdtd_version": ([], C.c_int),
    "fdtd_status_string": ([C.c_int], C.c_char_p),
    "fdtd_last_cuda_error": ([], C.c_int),
    "fdtd_status_to_error": ([C.c_int], C.c_int),
    "fdtd2d_dfield": ([C.c_int, C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_efield": ([C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_hfield": ([C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_ezinct": ([C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_inctdz": ([C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_hxinct": ([C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_incth": ([C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_fourier": ([C.c_int, C.POINTER(Params2D), C.POINTER(State2D), P], C.c_int),
    "fdtd2d_workspace_size": ([C.POINTER(Params2D), C.c_int], C.c_size_t),
    "fdtd2d_step_n": ([C.POINTER(Params2D), C.POINTER(State2D), C.c_int, C.c_int, C.c_int, P, C.c_size_t, P],
                      C.c_int),
    "fdtd2d_set_march_config": ([C.c_int, C.c_int, C.c_int], C.c_int),
    "fdtd2d_set_march_balance": ([C.c_float], C.c_int),
    "fdtd2d_pass": ([C.POINTER(Params2D), C.POINTER(Fields2D), C.POINTER(Fields2D), F, C.c_int, C.c_int, P, P],
                    C.c_int),
    "fdtd2d_adjoint_step": ([C.c_int, C.POINTER(Params2D), C.POINTER(Fields2D), C.POINTER(Fields2D), F, C.c_int,
                             C.c_int, C.c_float, Box2D, F, F, P], C.c_int),
    "fdtd2d_tm_adjoint_workspace_size": ([C.POINTER(Params2D), C.POINTER(AdjointParams2D)], C.c_size_t),
    "fdtd2d_tm_adjoint_forward": ([C.POINTER(Params2D), C.POINTER(AdjointParams2D), F, P, P, C.c_size_t, P],
                                  C.c_int),
    "fdtd2d_tm_adjoint_reverse": ([C.POINTER(Params2D), C.POINTER(AdjointParams2D), F, F, P, C.c_size_t, P],
                                  C.c_int),
    "fdtd2d_tm_adjoint": ([C.POINTER(Params2D), C.POINTER(AdjointParams2D), F, P, F, F, P, C.c_size_t, P], C.c_int),
    "fno_profile_features": ([C.c_int, P, P, P, P, P, P, C.c_int, C.c_double, C.c_double, F, P], C.c_int),
    "fdtd_dft_amplitude_phase": ([C.c_int, C.c_longlong, F, F, C.c_longlong, F, F, P, P, P], C.c_int),
    "fdtd2d_step_n_noalloc": ([C.POINTER(Params2D), C.POINTER(State2D), C.c_int, C.c_int, C.c_int, P], C.c_int),
    "fdtd2d_dielectric_cylinder": ([C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                    F, F, P], C.c_int),
    "fdtd_check_finite": ([F, C.c_size_t, P, P], C.c_int),
    "fdtd1d_efield": ([C.c_int, C.POINTER(Params1D), C.POINTER(State1D), P], C.c_int),
    "fdtd1d_hfield": ([C.POINTER(Params1D), C.POINTER(State1D), P], C.c_int),
    "fdtd1d_fourier": ([C.c_int, C.POINTER(Params1D), C.POINTER(State1D), P], C.c_int),
    "fdtd1d_step_n": ([C.POINTER(Params1D), C.POINTER(State1D), C.c_int, C.c_int, P], C.c_int),
    "fdtd_gemm_bf16": ([C.POINTER(GemmDesc), P, P], C.c_int),
    "fno_lift_fwd": ([C.c_longlong, C.c_int, C.c_int, F, F, F, P, P], C.c_int),
    "fno_lift_bwd": ([C.c_longlong, C.c_int, C.c_int, F, P, F, F, P], C.c_int),
    "fno_propagation": ([C.c_int, C.c_int, F, C.c_int, P, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, F, P],
                        C.c_int),
    "fno_cmul": ([C.c_longlong, C.c_int, F, F, C.c_int, F, P], C.c_int),
    "fno_dft_to_modes": ([C.c_int, C.c_int, C.c_int, F, P, P], C.c_int),
    "fno_modes_to_dft": ([C.c_int, C.c_int, C.c_int, F, P, P], C.c_int),
    "fno_build_rbig": ([C.c_int, C.c_int, F, F, P, P], C.c_int),
    "fno_fold_drbig": ([C.c_int, C.c_int, F, F, F, P], C.c_int),
    "fno_pack_inputs": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, F, P, P, P], C.c_int),
    "fno_small_matmul": ([C.c_int, C.c_int, C.c_int, C.c_int, F, F, F, P], C.c_int),
    "fno_build_rbig_rect": ([C.c_int, C.c_int, C.c_int, F, F, P, P], C.c_int),
    "fno_gelu_fwd": ([C.c_longlong, F, P, P, P], C.c_int),
    "fno_gelu_bwd": ([C.c_longlong, P, F, P, P, P], C.c_int),
    "fno_meanpool": ([C.c_int, C.c_int, C.c_int, P, P, P], C.c_int),
    "fno_meanpool_bwd": ([C.c_int, C.c_int, C.c_int, F, P, P], C.c_int),
    "fno_colsum": ([C.c_longlong, C.c_int, P, F, F, P], C.c_int),
    "fno_sum_parts": ([C.c_int, C.c_longlong, F, F, P], C.c_int),
    "fno_mse": ([C.c_int, C.c_int, F, F, F, F, P], C.c_int),
    "fno_rel_mse": ([C.c_int, C.c_int, C.c_float, F, F, F, F, P], C.c_int),
    "fno_adam": ([C.c_longlong, F, F, F, F, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, P, P], C.c_int),
    "fno_to_bf16": ([C.c_longlong, F, P, P], C.c_int),
    "fdtd1d_batch_plan": ([P, C.c_int, C.c_int, C.c_int, P, C.c_size_t, C.POINTER(C.c_int)], C.c_int),
    "fdtd1d_batch_run": ([C.POINTER(BatchParams1D), C.POINTER(BatchOut1D), P, C.c_int, C.c_int, C.c_int, C.c_int,
                          C.c_int, C.c_longlong, P], C.c_int),
}

_LIB = None


def lib_path() -> str:
    return os.environ.get("FDTD_GB300_LIB", LIB)


def lib():
    """Load (once) and return the ctypes handle; raises if the library is absent."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise FdtdLibraryError(
                f"{path} is missing: build it with `python -m simulation_gb300.build` "
                "(the CUDA library is the only compute path)")
        try:
            h = C.CDLL(path)
        except OSError as e:
            raise FdtdLibraryError(f"cannot load {path}: {e}") from e
        for name, (args, res) in _SIGS.items():
            fn = getattr(h, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = h
    return _LIB


def declared_symbols() -> list[str]:
    return list(_SIGS)


def call(name: str, *args) -> int:
    rc = getattr(lib(), name)(*args)
    if rc != FDTD_OK:
        raise FdtdError(rc, name)
    return rc


def ptr(t) -> int | None:
    """Device address of a torch tensor (None for None)."""
    if t is None:
        return None
    return t.data_ptr()


def stream_ptr(stream=None) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
