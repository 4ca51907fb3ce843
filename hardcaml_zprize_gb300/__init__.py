"""GB300 Pippenger MSM engine for BLS12-377 G1 -- Python host mirror of the reference harness.

The product is ``libdriver.so`` (CUDA for sm_103a behind the C ABI in include/msm_gb300.h).
This module binds it with ctypes and mirrors the reference's Rust harness API
(zprize/msm_pippenger/test_fpga_harness/src/lib.rs:40-85):

    ctx = multi_scalar_mult_init(points)            # load the bases once
    out = multi_scalar_mult(ctx, points, scalars)   # batch = len(scalars) // len(points)

with the same argument meaning and the same error behaviour ("length mismatch" when the scalar
count is not a multiple of the point count, lib.rs:65-67).  Points are arrays of the 104-byte
``g1_affine_t`` records, scalars arrays of 4 x u64, results arrays of 144-byte
``g1_projective_t`` records (rust_types.h:8-83).

There is no CPU fallback: when the library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libdriver.so")

AFFINE_BYTES = 104
PROJ_BYTES = 144
SCALAR_BYTES = 32

# every symbol include/msm_gb300.h declares
EXPORTED = [
    "msm_init", "msm_mult", "msm_last_error", "msm_free", "msm_mult_ex", "msm_mult_uneven",
    "msm_mult_device", "msm_get_config", "msm_context_info", "msm_tune_uneven", "msm_tuned_form", "msm_tune", "msm_set_timing", "msm_last_timings",
    "msm_last_pass_stats", "msm_server_create", "msm_server_submit", "msm_server_poll",
    "msm_server_stats", "msm_server_destroy", "msm_generate_bases", "msm_generate_scalars",
    "msm_measure_imad_peak", "msm_device_info", "msm_field_selftest", "msm_measure_madd_rate",
    "msm_mult_noalloc", "msm_measure_int_peaks", "msm_fq_to_montgomery", "msm_fq_from_montgomery",
    "msm_fr_to_montgomery", "msm_fr_from_montgomery",
    "zprize_msm_fpga_init", "zprize_msm_fpga_mult", "zprize_msm_pippenger_mult",
]

STAGES = ["count", "scan", "scatter", "tasks", "accumulate", "merge", "reduce1", "reduce2",
          "reduce3", "final"]


class MsmOptions(ctypes.Structure):
    _fields_ = [("window_bits", ctypes.c_int32), ("signed_digits", ctypes.c_int32),
                ("seg_len", ctypes.c_int32), ("red_len_log2", ctypes.c_int32),
                ("use_graph", ctypes.c_int32), ("mode", ctypes.c_int32),
                ("fixed_base", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("passes", ctypes.c_uint64), ("inflight_peak", ctypes.c_uint64),
                ("bytes_in_use", ctypes.c_uint64), ("bytes_peak", ctypes.c_uint64)]


class MsmError(RuntimeError):
    pass


_lib: Optional[ctypes.CDLL] = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libdriver.so and declare its signatures; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise MsmError(f"{path} is missing: build it with `python -m hardcaml_zprize_gb300.build`")
    lib = ctypes.CDLL(path)
    P, U64, I32, I64, SZ = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t
    sig = {
        "msm_init": (P, [P, ctypes.c_ssize_t, P, ctypes.c_ssize_t]),
        "msm_mult": (None, [P, P, U64, P]),
        "zprize_msm_fpga_init": (P, [P, ctypes.c_ssize_t]),
        "zprize_msm_fpga_mult": (None, [P, P, U64, P]),
        "zprize_msm_pippenger_mult": (None, [P, P, U64, P]),
        "msm_last_error": (ctypes.c_int, [ctypes.c_char_p, SZ]),
        "msm_free": (None, [P]),
        "msm_mult_ex": (ctypes.c_int, [P, P, U64, P, ctypes.POINTER(MsmOptions)]),
        "msm_mult_uneven": (ctypes.c_int, [P, P, U64, P, P, P, ctypes.POINTER(MsmOptions)]),
        "msm_mult_device": (ctypes.c_int, [P, P, U64, P, P, P, ctypes.POINTER(MsmOptions)]),
        "msm_get_config": (ctypes.c_int, [P, U64, ctypes.POINTER(MsmOptions)]),
        "msm_context_info": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_uint64), I32]),
        "msm_tune_uneven": (ctypes.c_int, [P, U64, P, P, P, I32, ctypes.POINTER(MsmOptions),
                                           ctypes.POINTER(ctypes.c_double)]),
        "msm_tuned_form": (ctypes.c_int, [P, U64, I32, ctypes.POINTER(MsmOptions)]),
        "msm_tune": (ctypes.c_int, [P, U64, I32, ctypes.POINTER(MsmOptions)]),
        "msm_set_timing": (ctypes.c_int, [P, I32]),
        "msm_last_timings": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_double), I32]),
        "msm_last_pass_stats": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_uint64), I32]),
        "msm_server_create": (P, [P, U64, I32]),
        "msm_server_submit": (I64, [P, P, U64, U64]),
        "msm_server_poll": (ctypes.c_int, [P, I64, P, I32, ctypes.POINTER(ctypes.c_double)]),
        "msm_server_stats": (ctypes.c_int, [P, ctypes.POINTER(ServerStats)]),
        "msm_server_destroy": (None, [P]),
        "msm_generate_bases": (ctypes.c_int, [U64, U64, U64, P]),
        "msm_generate_scalars": (ctypes.c_int, [U64, U64, I32, U64, P]),
        "msm_measure_imad_peak": (ctypes.c_double, [I32]),
        "msm_device_info": (ctypes.c_int, [ctypes.c_char_p, SZ]),
        "msm_field_selftest": (ctypes.c_int, [I32, P, P, P, U64]),
        "msm_measure_madd_rate": (ctypes.c_double, [P, I32]),
        "msm_mult_noalloc": (ctypes.c_int, [P, P, U64, U64, P, P]),
        "msm_measure_int_peaks": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), I32]),
        "msm_fq_to_montgomery": (ctypes.c_int, [P, U64]),
        "msm_fq_from_montgomery": (ctypes.c_int, [P, U64]),
        "msm_fr_to_montgomery": (ctypes.c_int, [P, U64]),
        "msm_fr_from_montgomery": (ctypes.c_int, [P, U64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    lib = load_library()
    buf = ctypes.create_string_buffer(512)
    code = lib.msm_last_error(buf, 512)
    return f"[{code}] {buf.value.decode(errors='replace')}"


def _check(rc: int, what: str):
    if rc != 0:
        raise MsmError(f"{what}: {last_error()}")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def as_points(points) -> np.ndarray:
    a = np.ascontiguousarray(np.frombuffer(points, dtype=np.uint8) if isinstance(points, (bytes, bytearray)) else points, dtype=np.uint8)
    if a.size % AFFINE_BYTES:
        raise ValueError("points must be whole 104-byte g1_affine_t records")
    return a.reshape(-1, AFFINE_BYTES)


def as_scalars(scalars) -> np.ndarray:
    a = np.ascontiguousarray(np.frombuffer(scalars, dtype=np.uint64) if isinstance(scalars, (bytes, bytearray)) else scalars, dtype=np.uint64)
    if a.size % 4:
        raise ValueError("scalars must be whole 4 x u64 records")
    return a.reshape(-1, 4)


def _opts(**kw) -> Optional[MsmOptions]:
    if not kw:
        return None
    o = MsmOptions()
    for k, v in kw.items():
        setattr(o, k, int(v))
    return o


class MultiScalarMultContext:
    """Owns a device context (lib.rs:35-38 keeps a raw pointer; this one frees on close)."""

    def __init__(self, handle: int, npoints: int):
        self.handle = handle
        self.npoints = npoints

    def close(self):
        if self.handle:
            load_library().msm_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- additions beyond the reference harness ---
    def mult(self, scalars, **opts) -> np.ndarray:
        sc = as_scalars(scalars)
        n = max(self.npoints, 1)
        if self.npoints == 0 or sc.shape[0] % n:
            raise ValueError("length mismatch")
        batch = sc.shape[0] // n
        out = np.zeros((batch, PROJ_BYTES), dtype=np.uint8)
        o = _opts(**opts)
        _check(load_library().msm_mult_ex(self.handle, _ptr(out), batch, _ptr(sc),
                                          ctypes.byref(o) if o else None), "msm_mult_ex")
        return out

    def mult_uneven(self, sizes: Sequence[int], offsets: Sequence[int], scalars, **opts) -> np.ndarray:
        sc = as_scalars(scalars)
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        of = np.ascontiguousarray(offsets, dtype=np.uint64)
        if sc.shape[0] != int(sz.sum()):
            raise ValueError("length mismatch")
        out = np.zeros((len(sz), PROJ_BYTES), dtype=np.uint8)
        o = _opts(**opts)
        _check(load_library().msm_mult_uneven(self.handle, _ptr(out), len(sz), _ptr(sz), _ptr(of),
                                              _ptr(sc), ctypes.byref(o) if o else None),
               "msm_mult_uneven")
        return out

    def mult_device(self, sizes, offsets, d_scalars_ptr: int, **opts) -> np.ndarray:
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        of = np.ascontiguousarray(offsets, dtype=np.uint64)
        out = np.zeros((len(sz), PROJ_BYTES), dtype=np.uint8)
        o = _opts(**opts)
        _check(load_library().msm_mult_device(self.handle, _ptr(out), len(sz), _ptr(sz), _ptr(of),
                                              ctypes.c_void_p(d_scalars_ptr),
                                              ctypes.byref(o) if o else None), "msm_mult_device")
        return out

    def config(self, n: int) -> dict:
        o = MsmOptions()
        _check(load_library().msm_get_config(self.handle, n, ctypes.byref(o)), "msm_get_config")
        return {f: getattr(o, f) for f, _ in MsmOptions._fields_}

    def info(self) -> dict:
        """What the context keeps resident: bases, bytes of base records, table sets."""
        arr = (ctypes.c_uint64 * 6)()
        k = load_library().msm_context_info(self.handle, arr, 6)
        if k < 0:
            raise MsmError(f"msm_context_info: {last_error()}")
        keys = ["npoints", "resident_bytes", "table_bits", "table_windows", "table2_bits",
                "table2_windows"]
        return {keys[i]: int(arr[i]) for i in range(k)}

    def tune(self, n: int, budget_ms: int = 0) -> dict:
        o = MsmOptions()
        _check(load_library().msm_tune(self.handle, n, budget_ms, ctypes.byref(o)), "msm_tune")
        return {f: getattr(o, f) for f, _ in MsmOptions._fields_}

    def tune_uneven(self, sizes: Sequence[int], offsets: Sequence[int], scalars,
                    budget_ms: int = 0) -> dict:
        """Tune the one-pass form on this batch (msm_tune_uneven).  Returns the pass-level options
        to pass back with the same mix (``opts``), the untuned and tuned pass times (ms) and the
        per-size-class forms now used in shared passes."""
        sc = as_scalars(scalars)
        sz = np.ascontiguousarray(sizes, dtype=np.uint64)
        of = np.ascontiguousarray(offsets, dtype=np.uint64)
        if sc.shape[0] != int(sz.sum()):
            raise ValueError("length mismatch")
        o = MsmOptions()
        rep = (ctypes.c_double * 3)()
        _check(load_library().msm_tune_uneven(self.handle, len(sz), _ptr(sz), _ptr(of), _ptr(sc),
                                              budget_ms, ctypes.byref(o), rep), "msm_tune_uneven")
        opts = {f: getattr(o, f) for f, _ in MsmOptions._fields_ if getattr(o, f)}
        classes = sorted({(max(int(x), 1) - 1).bit_length() for x in sz})  # ceil(log2 n)
        forms = {c: self.tuned_form(1 << c, shared_pass=True) for c in classes}
        return {"opts": opts, "untuned_ms": rep[0], "tuned_ms": rep[1], "passes_measured": int(rep[2]),
                "forms": forms}

    def tuned_form(self, n: int, shared_pass: bool = False) -> dict:
        """Window width, digit signs and the bases read (0 plain records, 1 main tables,
        2 width-16 tables) for an MSM of n points, alone or in a shared pass."""
        o = MsmOptions()
        _check(load_library().msm_tuned_form(self.handle, n, 1 if shared_pass else 0, ctypes.byref(o)),
               "msm_tuned_form")
        return {"window_bits": o.window_bits, "signed": o.signed_digits == 1, "bases": o.fixed_base}

    def set_timing(self, on: bool):
        _check(load_library().msm_set_timing(self.handle, 1 if on else 0), "msm_set_timing")

    def last_timings(self) -> dict:
        arr = (ctypes.c_double * len(STAGES))()
        n = load_library().msm_last_timings(self.handle, arr, len(STAGES))
        return {STAGES[k]: arr[k] for k in range(n)}

    def last_pass_stats(self) -> dict:
        arr = (ctypes.c_uint64 * 5)()
        load_library().msm_last_pass_stats(self.handle, arr, 5)
        return {"tasks": arr[0], "heavy_buckets": arr[1], "entries": arr[2], "buckets": arr[3],
                "kernels": arr[4]}

    def mult_noalloc(self, n: int, base_offset: int, d_scalars_ptr: int, d_out_ptr: int,
                     stream: int = 0) -> None:
        """Enqueue one MSM of n <= 65536 points that allocates no device memory: the caller
        passes device pointers for the scalars and the 144-byte result and synchronises."""
        _check(load_library().msm_mult_noalloc(self.handle, ctypes.c_void_p(d_out_ptr), n,
                                               base_offset, ctypes.c_void_p(d_scalars_ptr),
                                               ctypes.c_void_p(stream) if stream else None),
               "msm_mult_noalloc")

    def madd_rate(self, iters: int = 2000) -> float:
        return load_library().msm_measure_madd_rate(self.handle, iters)


def multi_scalar_mult_init(points) -> MultiScalarMultContext:
    """Mirror of lib.rs:40-57: load the bases once.  XCLBIN is read for parity but unused."""
    pts = as_points(points)
    xcl = os.environ.get("XCLBIN", "").encode()
    h = load_library().msm_init(xcl or None, len(xcl), _ptr(pts), pts.shape[0])
    if not h:
        raise MsmError(f"msm_init: {last_error()}")
    return MultiScalarMultContext(h, pts.shape[0])


def multi_scalar_mult(context: MultiScalarMultContext, points, scalars) -> np.ndarray:
    """Mirror of lib.rs:59-85: batch_size = len(scalars) / len(points), one result per batch."""
    npoints = as_points(points).shape[0]
    sc = as_scalars(scalars)
    if npoints == 0 or sc.shape[0] % npoints != 0:
        raise ValueError("length mismatch")
    batch = sc.shape[0] // npoints
    out = np.zeros((batch, PROJ_BYTES), dtype=np.uint8)
    load_library().msm_mult(context.handle, _ptr(out), batch, _ptr(sc))
    lib = load_library()
    buf = ctypes.create_string_buffer(512)
    if lib.msm_last_error(buf, 512) != 0:
        raise MsmError(f"msm_mult: {buf.value.decode(errors='replace')}")
    return out


# ---- utilities ------------------------------------------------------------------------------
def generate_bases(seed: int, n: int, first: int = 0) -> np.ndarray:
    """k_i * G for seeded 64-bit k_i, computed on the GPU (g1_affine_t records)."""
    out = np.zeros((n, AFFINE_BYTES), dtype=np.uint8)
    _check(load_library().msm_generate_bases(seed, first, n, _ptr(out)), "msm_generate_bases")
    return out


def generate_scalars(seed: int, n: int, kind: int = 0, msm_index: int = 0) -> np.ndarray:
    """Seeded scalars (kind 0 uniform in [0, r), kind 1 the uneven-batch mix), 4 x u64 each."""
    out = np.zeros((n, 4), dtype=np.uint64)
    _check(load_library().msm_generate_scalars(seed, n, kind, msm_index, _ptr(out)),
           "msm_generate_scalars")
    return out


def measure_imad_peak(iters: int = 20000) -> float:
    return load_library().msm_measure_imad_peak(iters)


def measure_int_peaks() -> dict:
    """IMAD-pipe rates (per second): mad.lo/mad.hi pairs, mad.lo only, mad.hi only."""
    arr = (ctypes.c_double * 3)()
    n = load_library().msm_measure_int_peaks(arr, 3)
    if n <= 0:
        raise MsmError(f"msm_measure_int_peaks: {last_error()}")
    return {"mad_lo_hi": arr[0], "mad_lo": arr[1], "mad_hi": arr[2]}


def device_info() -> str:
    buf = ctypes.create_string_buffer(256)
    _check(load_library().msm_device_info(buf, 256), "msm_device_info")
    return buf.value.decode()


def field_selftest(op: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint32).reshape(-1, 12)
    b = np.ascontiguousarray(b, dtype=np.uint32).reshape(-1, 12)
    out = np.zeros_like(a)
    _check(load_library().msm_field_selftest(op, _ptr(a), _ptr(b), _ptr(out), a.shape[0]),
           "msm_field_selftest")
    return out


class MsmServer:
    """Continuous-batching request loop over the resident bases (msm_server_* in the C ABI)."""

    def __init__(self, ctx: MultiScalarMultContext, hbm_budget_bytes: int, max_inflight: int = 2):
        self.ctx = ctx
        self.handle = load_library().msm_server_create(ctx.handle, hbm_budget_bytes, max_inflight)
        if not self.handle:
            raise MsmError(f"msm_server_create: {last_error()}")

    def submit(self, scalars, base_offset: int = 0) -> int:
        sc = as_scalars(scalars)
        rid = load_library().msm_server_submit(self.handle, _ptr(sc), sc.shape[0], base_offset)
        if rid < 0:
            raise MsmError(f"msm_server_submit: {last_error()}")
        return rid

    def poll(self, rid: int, wait_ms: int = 0):
        out = np.zeros(PROJ_BYTES, dtype=np.uint8)
        lat = ctypes.c_double(0)
        rc = load_library().msm_server_poll(self.handle, rid, _ptr(out), wait_ms, ctypes.byref(lat))
        if rc < 0:
            raise MsmError(f"msm_server_poll: {last_error()}")
        if rc == 1:
            return None
        return out, lat.value

    def stats(self) -> dict:
        st = ServerStats()
        _check(load_library().msm_server_stats(self.handle, ctypes.byref(st)), "msm_server_stats")
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if self.handle:
            load_library().msm_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
