"""ctypes binding of the CUDA library ``libqmprs_gb300.so`` (C ABI in
``include/qmprs_gb300.h``).

The library is built in-tree by ``qmprs_gb300.build``.  There is no CPU
fallback: loading fails loudly when the library is missing, and every call
that reaches it needs a CUDA device.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "_lib"
LIB_PATH = LIB_DIR / "libqmprs_gb300.so"

OK = 0
ERR_INVALID = 1
ERR_UNSUPPORTED = 2
ERR_CUDA = 3
ERR_NUMERIC = 4
ERR_NONUNITARY = 5

PRECISION_FAST = 0
PRECISION_EXACT = 1
PRECISIONS = {"fast": PRECISION_FAST, "exact": PRECISION_EXACT}

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)
_c_void_p = ctypes.c_void_p

# name -> (restype, argtypes); mirrors include/qmprs_gb300.h
SIGNATURES: dict[str, tuple] = {
    "qmprs_version": (ctypes.c_int, []),
    "qmprs_launch_count": (ctypes.c_int64, []),
    "qmprs_plan_set_profiling": (ctypes.c_int, [_c_void_p, ctypes.c_int]),
    "qmprs_plan_profile": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_i64_p, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "qmprs_create": (ctypes.c_int, [ctypes.POINTER(_c_void_p)]),
    "qmprs_destroy": (None, [_c_void_p]),
    "qmprs_last_error": (ctypes.c_char_p, [_c_void_p]),
    "qmprs_plan_create": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_int_p, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(_c_void_p)]),
    "qmprs_plan_destroy": (None, [_c_void_p]),
    "qmprs_plan_layout": (ctypes.c_int, [_c_void_p, _c_i64_p, _c_i64_p, _c_i64_p, _c_i64_p, _c_i64_p, _c_i64_p]),
    "qmprs_plan_max_qubits": (ctypes.c_int, [_c_void_p]),
    "qmprs_plan_set_precision": (ctypes.c_int, [_c_void_p, ctypes.c_int]),
    "qmprs_plan_precision": (ctypes.c_int, [_c_void_p]),
    "qmprs_plan_set_graphs": (ctypes.c_int, [_c_void_p, ctypes.c_int]),
    "qmprs_plan_graph_stats": (ctypes.c_int, [_c_void_p, _c_int_p, _c_i64_p]),
    "qmprs_plan_wide_stats": (ctypes.c_int, [_c_void_p, _c_int_p, _c_int_p, _c_int_p,
                                             ctypes.POINTER(ctypes.c_float)]),
    "qmprs_plan_set_autotune": (ctypes.c_int, [_c_void_p, ctypes.c_int]),
    "qmprs_plan_tuning": (ctypes.c_int, [_c_void_p, _c_int_p, _c_int_p]),
    "qmprs_plan_upload": (ctypes.c_int, [_c_void_p, _c_void_p, ctypes.c_int64, _c_void_p, ctypes.POINTER(_c_void_p)]),
    "qmprs_mps_from_statevector": (ctypes.c_int, [_c_void_p, _c_void_p, ctypes.c_int, ctypes.c_double, _c_void_p,
                                                  _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_mps_to_statevector": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_unitary_layers": (ctypes.c_int, [_c_void_p, _c_void_p, ctypes.c_int, ctypes.c_double, _c_void_p,
                                            _c_void_p, _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_optimize_layers": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, ctypes.c_int,
                                             ctypes.c_double, _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_layer_environments": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                                                _c_void_p]),
    "qmprs_circuit_state": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_overlap": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_apply_layer": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, ctypes.c_int, ctypes.c_int,
                                         _c_void_p]),
    "qmprs_overlap_noalloc": (ctypes.c_int, [_c_void_p, _c_void_p, ctypes.c_int, _c_int_p, _c_void_p, _c_void_p]),
    "qmprs_gemm_bf16": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, _c_void_p, _c_void_p, ctypes.c_int, ctypes.c_int,
                                       _c_void_p, ctypes.c_int, _c_void_p, _c_void_p, ctypes.c_int, _c_void_p,
                                       _c_void_p, _c_void_p]),
    "qmprs_mlp_loss": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, ctypes.c_int, ctypes.c_float, _c_void_p,
                                      _c_void_p, _c_void_p, _c_void_p, ctypes.c_int, _c_void_p]),
    "qmprs_mlp_act_back": (ctypes.c_int, [_c_void_p, _c_void_p, ctypes.c_int, ctypes.c_int, _c_void_p, _c_void_p,
                                          _c_void_p, ctypes.c_int, _c_void_p]),
    "qmprs_mlp_col_sum": (ctypes.c_int, [_c_void_p, ctypes.c_int, ctypes.c_int, _c_void_p, _c_void_p]),
    "qmprs_mlp_adam": (ctypes.c_int, [_c_void_p, _c_void_p, ctypes.c_int, _c_void_p, _c_void_p, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_int, ctypes.c_float, _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_mlp_project": (ctypes.c_int, [_c_void_p, ctypes.c_int, _c_void_p, _c_void_p, _c_void_p, _c_void_p]),
    "qmprs_tc_wait_selftest": (ctypes.c_int, [_c_void_p, _c_void_p]),
    "qmprs_mlp_overlap_grad": (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_float, _c_void_p, _c_void_p, _c_void_p,
                                              _c_void_p, ctypes.c_int, _c_void_p]),
}

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    """A CUDA-side failure (launch error, unsupported size, numerical failure)."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def load() -> ctypes.CDLL:
    """Load the CUDA library (once).  Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m qmprs_gb300.build` "
                "(qmprs_gb300 has no CPU fallback)")
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def raise_for(code: int, handle) -> None:
    """Map a status code to the reference's exception classes."""
    if code == OK:
        return
    msg = load().qmprs_last_error(handle)
    text = msg.decode() if msg else f"error {code}"
    if code in (ERR_INVALID, ERR_NONUNITARY):
        raise ValueError(text)
    raise NativeError(code, text)
