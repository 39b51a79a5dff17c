"""GB300-native TeaLeaf CG backend: Python bindings of the C ABI.

The product is the CUDA library ``_build/libtealeaf_gb300.so`` (C ABI in
``include/tealeaf_gb300.h``) and the TeaLeaf driver built on it
(``_build/tealeaf_gb300``). This module loads the library with ctypes and
offers a thin ``Context`` for device fields; it has no compute of its own
and no fallback: if the library is missing or no GPU is usable, every call
raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
BUILD = PKG / "_build"
LIB_PATH = BUILD / "libtealeaf_gb300.so"
DRIVER_EXE = BUILD / "tealeaf_gb300"

TL_OK = 0
# Largest grid (x*y cells, halos included): TL_MAX_CELLS of include/tealeaf_gb300.h.
MAX_CELLS = 536_870_912
TL_ERRORS = {1: "TL_ERR_CUDA", 2: "TL_ERR_ARG", 3: "TL_ERR_TIMEOUT", 4: "TL_ERR_STATE",
             5: "TL_ERR_NUMERIC"}

RECTANGULAR, CIRCULAR, POINT = 0, 1, 2
CHUNK_LEFT, CHUNK_RIGHT, CHUNK_BOTTOM, CHUNK_TOP = 0, 1, 2, 3
CONDUCTIVITY, RECIP_CONDUCTIVITY = 1, 2


class TLError(RuntimeError):
    """A C-ABI call returned an error code."""


class TLSolveStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_float), ("steps", C.c_int), ("kernel_launches", C.c_int)]


class TLSolveParams(C.Structure):
    _fields_ = [("method", C.c_int), ("rel_tol", C.c_double), ("inner_tol", C.c_double),
                ("max_inner", C.c_int), ("max_outer", C.c_int), ("stall_factor", C.c_double),
                ("max_fallback", C.c_int), ("learned", C.c_void_p), ("projection", C.c_int)]


class TLSolveReport(C.Structure):
    _fields_ = [("outer_steps", C.c_int), ("inner_steps", C.c_int),
                ("fallback_events", C.c_int), ("fallback_steps", C.c_int),
                ("initial_rel_residual", C.c_double), ("final_rel_residual", C.c_double),
                ("device_ms", C.c_float), ("inner_kernel_ms", C.c_float),
                ("projection_basis", C.c_int)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


METHOD_CG64, METHOD_MIXED_CG, METHOD_MIXED_JACOBI, METHOD_MIXED_LEARNED = 0, 1, 2, 3
METHOD_MIXED_LEARNED_LAYERS = 4
METHOD_MIXED_LEARNED_COARSE = 5
FP64_CONTRACTS = {"exact": 0, "fused": 1}
METHODS = {"cg64": METHOD_CG64, "mixed": METHOD_MIXED_CG, "mixed-jacobi": METHOD_MIXED_JACOBI,
           "mixed-learned": METHOD_MIXED_LEARNED,
           "mixed-learned-layers": METHOD_MIXED_LEARNED_LAYERS,
           "mixed-learned-coarse": METHOD_MIXED_LEARNED_COARSE}


class TLState(C.Structure):
    _fields_ = [("density", C.c_double), ("energy", C.c_double), ("x_min", C.c_double),
                ("y_min", C.c_double), ("x_max", C.c_double), ("y_max", C.c_double),
                ("radius", C.c_double), ("geometry", C.c_int)]


_P = C.c_void_p          # device pointer / opaque handle
_D = C.c_double
_I = C.c_int
_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int)

# name -> argument types after the context argument (all return int).
SIGNATURES: dict[str, list] = {
    "tl_set_chunk_data_vertices": [_I, _I, _I, _P, _P, _D, _D, _D, _D],
    "tl_set_chunk_data": [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _D, _D, _D, _D],
    "tl_set_chunk_initial_state": [_I, _I, _D, _D, _P, _P],
    "tl_set_chunk_state": [_I, _I, _I, C.POINTER(TLState), _P, _P, _P, _P, _P, _P, _P],
    "tl_store_energy": [_I, _I, _P, _P],
    "tl_update_face": [_I, _I, _I, _P, _I, _I],
    "tl_local_halos": [_I, _I, _I, _I, _I, C.POINTER(C.c_void_p), _I],
    "tl_pack_or_unpack": [_I, _I, _I, _I, _I, _I, _P, _PD],
    "tl_field_summary": [_I, _I, _I, _P, _P, _P, _P, _PD, _PD, _PD, _PD],
    "tl_cg_init": [_I, _I, _I, _I, _D, _D, _P, _P, _P, _P, _P, _P, _P, _P, _PD],
    "tl_cg_calc_w": [_I, _I, _I, _P, _P, _P, _P, _PD],
    "tl_cg_calc_ur": [_I, _I, _I, _P, _P, _P, _P, _D, _PD],
    "tl_cg_calc_p": [_I, _I, _I, _D, _P, _P],
    "tl_cg_solve": [_I, _I, _I, _I, _D, _D, _D, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                    _PD, _PD, _PD, _PI],
    "tl_copy_u": [_I, _I, _I, _P, _P],
    "tl_calculate_residual": [_I, _I, _I, _P, _P, _P, _P, _P],
    "tl_calculate_2norm": [_I, _I, _I, _P, _PD],
    "tl_finalise": [_I, _I, _I, _P, _P, _P],
    "tl_jacobi_init": [_I, _I, _I, _I, _D, _D, _P, _P, _P, _P, _P, _P],
    "tl_jacobi_iterate": [_I, _I, _I, _P, _P, _P, _P, _P, _PD],
    "tl_cheby_init": [_I, _I, _I, _D, _P, _P, _P, _P, _P, _P, _P],
    "tl_cheby_iterate": [_I, _I, _I, _D, _D, _P, _P, _P, _P, _P, _P, _P],
    "tl_ppcg_init": [_I, _I, _I, _D, _P, _P],
    "tl_ppcg_inner_iteration": [_I, _I, _I, _D, _D, _D, _P, _P, _P, _P, _P],
    "tl_solve": [_I, _I, _I, _I, _D, _D, C.POINTER(TLSolveParams), _P, _P, _P, _P, _P, _P, _P,
                 _P, _P, C.POINTER(TLSolveReport)],
    "tl_projection_reset": [],
}

# Entry points that do not take a context first.
CONTEXT_FREE = {
    "tl_context_create": [_I, _P, C.POINTER(C.c_void_p)],
    "tl_context_destroy": [_P],
    "tl_context_stream": [_P, C.POINTER(C.c_void_p)],
    "tl_synchronize": [_P],
    "tl_field_alloc": [_P, C.c_size_t, C.POINTER(C.c_void_p)],
    "tl_field_free": [_P, _P],
    "tl_copy_to_device": [_P, _P, _P, C.c_size_t],
    "tl_copy_to_host": [_P, _P, _P, C.c_size_t],
    "tl_last_solve_stats": [_P, C.POINTER(TLSolveStats)],
    "tl_set_fp64_contract": [_P, _I],
    "tl_cg_calc_w_noalloc": [_P, _I, _I, _I, _P, _P, _P, _P, _PD],
    "tl_selftest_barrier_timeout": [_P, _I, _PI],
}

# Entry points whose first argument is a network or context handle (prepended).
HANDLE_FIRST = {
    "tl_net_create": [C.POINTER(C.c_void_p)],
    "tl_net_destroy": [],
    "tl_net_set_weights": [C.POINTER(C.c_float), _I],
    "tl_net_get_weights": [C.POINTER(C.c_float), _I],
    "tl_net_apply": [_I, _I, _I, _P, _P, _P],
    "tl_net_loss_grad": [_I, _I, _I, _I, _P, _P, _P, _P, _PD, C.POINTER(C.c_float)],
    "tl_net_adam_step": [C.c_float],
    "tl_net_stencil": [C.POINTER(C.c_float), C.POINTER(C.c_float)],
    "tl_net_apply_stencil": [_I, _I, _P, _P, _P],
    "tl_net_pcg": [_I, _I, _P, _P, _P, _P, _P, _D, _I, _PI, _PD],
    "tl_net_gather_crops": [_P, _I, _I, C.POINTER(C.c_int), _I, _I, _I, _P],
    "tl_pack_interior": [_I, _I, _I, _P, _D, _P],
    "tl_pack_coefficients": [_I, _I, _I, _P, _P, _P, _P, _P],
    "tl_coarse_inverse": [_I, _I, _P, _P, _PI, _PI, C.POINTER(C.c_float), C.c_size_t],
    "tl_coarse_inverse_f16": [_I, _I, _P, _P, C.POINTER(C.c_uint16), C.c_size_t, _PI],
}

_lib = None


def load_library(path: Path | None = None) -> C.CDLL:
    """Loads libtealeaf_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise TLError(f"{p} is missing: run exploringsycl_gb300.build.build_all() first")
    lib = C.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = [_P, *args]
        fn.restype = _I
    for name, args in CONTEXT_FREE.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _I
    for name, args in HANDLE_FIRST.items():
        fn = getattr(lib, name)
        fn.argtypes = [_P, *args]
        fn.restype = _I
    lib.tl_last_error.argtypes = []
    lib.tl_last_error.restype = C.c_char_p
    lib.tl_launch_count.argtypes = [_P]
    lib.tl_launch_count.restype = C.c_longlong
    lib.tl_net_num_params.argtypes = []
    lib.tl_net_num_params.restype = _I
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    if rc != TL_OK:
        msg = load_library().tl_last_error().decode(errors="replace")
        raise TLError(f"{what or 'call'} failed with {TL_ERRORS.get(rc, rc)}: {msg}")


def declared_symbols() -> list[str]:
    """Every entry point declared in include/tealeaf_gb300.h."""
    import re
    text = (PKG.parent / "include" / "tealeaf_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|long long)\s+(tl_\w+)\(", text,
                                 re.M)))


class Context:
    """A backend context (stream + scratch) and helpers for device fields."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load_library()
        self.h = C.c_void_p()
        check(self.lib.tl_context_create(device, stream, C.byref(self.h)), "tl_context_create")
        self._fields: list[int] = []

    def set_fp64_contract(self, contract: str) -> None:
        """'exact' (default) or 'fused': the arithmetic of the persistent
        FP64 CG solve (see tl_set_fp64_contract)."""
        check(self.lib.tl_set_fp64_contract(self.h, FP64_CONTRACTS[contract]),
              "tl_set_fp64_contract")

    # -- memory
    def alloc(self, n: int) -> int:
        p = C.c_void_p()
        check(self.lib.tl_field_alloc(self.h, n, C.byref(p)), "tl_field_alloc")
        self._fields.append(p.value)
        return p.value

    def alloc_f32(self, n: int) -> int:
        """Zeroed device array of n floats (allocated as doubles)."""
        return self.alloc((n + 1) // 2)

    def download_f32(self, dev: int, n: int) -> np.ndarray:
        out = np.empty((n + 1) // 2, dtype=np.float64)
        check(self.lib.tl_copy_to_host(self.h, out.ctypes.data, dev, out.size), "download")
        return out.view(np.float32)[:n].copy()

    def upload_f32(self, dev: int, host: np.ndarray) -> None:
        a = np.ascontiguousarray(host, dtype=np.float32).ravel()
        if a.size % 2:
            a = np.concatenate([a, np.zeros(1, np.float32)])
        check(self.lib.tl_copy_to_device(self.h, dev, a.ctypes.data, a.size // 2), "upload")

    def upload(self, dev: int, host: np.ndarray) -> None:
        a = np.ascontiguousarray(host, dtype=np.float64)
        check(self.lib.tl_copy_to_device(self.h, dev, a.ctypes.data, a.size), "upload")

    def download(self, dev: int, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.float64)
        check(self.lib.tl_copy_to_host(self.h, out.ctypes.data, dev, n), "download")
        return out

    def field_from(self, host: np.ndarray) -> int:
        dev = self.alloc(host.size)
        self.upload(dev, host)
        return dev

    def stream(self) -> int:
        s = C.c_void_p()
        check(self.lib.tl_context_stream(self.h, C.byref(s)), "tl_context_stream")
        return s.value or 0

    def synchronize(self) -> None:
        check(self.lib.tl_synchronize(self.h), "tl_synchronize")

    def solve_stats(self) -> TLSolveStats:
        st = TLSolveStats()
        check(self.lib.tl_last_solve_stats(self.h, C.byref(st)), "tl_last_solve_stats")
        return st

    def launches(self) -> int:
        return int(self.lib.tl_launch_count(self.h))

    # -- generic call: tl_<name>(ctx, *args)
    def call(self, name: str, *args) -> None:
        check(getattr(self.lib, name)(self.h, *args), name)

    def close(self) -> None:
        if self.h:
            for f in self._fields:
                self.lib.tl_field_free(self.h, f)
            self._fields.clear()
            check(self.lib.tl_context_destroy(self.h), "tl_context_destroy")
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


__all__ = ["Context", "TLError", "TLState", "load_library", "check", "declared_symbols",
           "LIB_PATH", "DRIVER_EXE"]
