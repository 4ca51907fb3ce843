"""NTT over the Goldilocks field on the GPU -- Python binding of the ntt_* entry points of
libdriver.so (include/ntt_gb300.h).

The transform is the reference's NTT track (zprize/ntt/host/reference.cpp:94-139): natural order
in and out, root of unity from zprize/ntt/host/gf.h:65-99.  It mirrors the calls the reference's
host programs make on their driver (simple_evaluate, input_vector_size).  There is no CPU
fallback: without the library or a GPU, calls raise.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import MsmError, load_library

GL_P = 0xFFFFFFFF00000001
EXPORTED = ["ntt_init", "ntt_init_inverse", "ntt_input_vector_size", "ntt_evaluate",
            "ntt_evaluate_device", "ntt_last_timings", "ntt_last_error", "ntt_free",
            "ntt_field_selftest", "ntt_evaluate_batch"]
NTT_STAGES = ["h2d", "pass_a", "pass_b", "d2h"]

_declared = False


def _lib():
    global _declared
    lib = load_library()
    if not _declared:
        P, U64, I32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32
        sig = {
            "ntt_init": (P, [ctypes.c_uint32]),
            "ntt_init_inverse": (P, [ctypes.c_uint32]),
            "ntt_input_vector_size": (U64, [P]),
            "ntt_evaluate": (ctypes.c_int, [P, P, P, U64]),
            "ntt_evaluate_device": (ctypes.c_int, [P, P, P, P]),
            "ntt_last_timings": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_double), I32]),
            "ntt_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
            "ntt_free": (None, [P]),
            "ntt_field_selftest": (ctypes.c_int, [I32, P, P, P, U64]),
            "ntt_evaluate_batch": (ctypes.c_int, [P, P, P, U64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _declared = True
    return lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(512)
    code = _lib().ntt_last_error(buf, 512)
    return f"[{code}] {buf.value.decode(errors='replace')}"


def field_selftest(op: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Element-wise a + b (op 0), a - b (1) or a b (2) modulo p on the GPU."""
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    out = np.empty_like(a)
    if _lib().ntt_field_selftest(op, a.ctypes.data, b.ctypes.data, out.ctypes.data, a.size) != 0:
        raise MsmError(f"ntt_field_selftest: {last_error()}")
    return out


class NttContext:
    """Transforms of 2^log_n points (log_n <= 24) with device buffers allocated once.  With
    inverse=True the context computes the inverse transform, x[j] = (1/n) sum_k X[k] w^(-j k)
    (ntt_init_inverse)."""

    def __init__(self, log_n: int, inverse: bool = False):
        self.handle = (_lib().ntt_init_inverse if inverse else _lib().ntt_init)(log_n)
        if not self.handle:
            raise MsmError(f"ntt_init: {last_error()}")
        self.inverse = inverse
        self.log_n = log_n
        self.n = 1 << log_n

    def input_vector_size(self) -> int:
        return int(_lib().ntt_input_vector_size(self.handle))

    def evaluate(self, values, out: Optional[np.ndarray] = None) -> np.ndarray:
        """NTT of host values (the reference's simple_evaluate)."""
        x = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1)
        if x.shape[0] != self.n:
            raise ValueError("length mismatch")
        if out is None:
            out = np.empty_like(x)
        if _lib().ntt_evaluate(self.handle, out.ctypes.data, x.ctypes.data, self.n) != 0:
            raise MsmError(f"ntt_evaluate: {last_error()}")
        return out

    def evaluate_batch(self, values, out: Optional[np.ndarray] = None) -> np.ndarray:
        """NTTs of several vectors (rows of `values`), transfers overlapping the transforms."""
        x = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1, self.n)
        if out is None:
            out = np.empty_like(x)
        if _lib().ntt_evaluate_batch(self.handle, out.ctypes.data, x.ctypes.data, x.shape[0]) != 0:
            raise MsmError(f"ntt_evaluate_batch: {last_error()}")
        return out

    def evaluate_device(self, d_out: int, d_in: int, stream: int = 0) -> None:
        """Enqueue the transform between device buffers (pointers); the caller synchronises."""
        rc = _lib().ntt_evaluate_device(self.handle, ctypes.c_void_p(d_out), ctypes.c_void_p(d_in),
                                        ctypes.c_void_p(stream) if stream else None)
        if rc != 0:
            raise MsmError(f"ntt_evaluate_device: {last_error()}")

    def last_timings(self) -> dict:
        arr = (ctypes.c_double * 4)()
        k = _lib().ntt_last_timings(self.handle, arr, 4)
        return {NTT_STAGES[i]: arr[i] for i in range(k)}

    def close(self):
        if self.handle:
            _lib().ntt_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
