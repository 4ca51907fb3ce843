"""ctypes bridge to the C oracle (oracle/cpu_msm.c) -- test infrastructure only.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker and the
timed CPU baseline; the GPU engine never calls it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def lib():
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        L = ctypes.CDLL(path)
        P, U64, I = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        L.oracle_msm.argtypes = [P, P, U64, I, I, P]
        L.oracle_msm.restype = I
        L.oracle_gen_bases.argtypes = [U64, U64, U64, P, I]
        L.oracle_gen_bases.restype = I
        L.oracle_mul.argtypes = [P, P, P]
        L.oracle_mul.restype = I
        L.oracle_default_window.argtypes = [U64]
        L.oracle_default_window.restype = I
        L.oracle_rand_u64.argtypes = [U64, U64, U64, U64]
        L.oracle_rand_u64.restype = U64
        L.oracle_gen_scalars.argtypes = [U64, U64, I, U64, P, I]
        L.oracle_gen_scalars.restype = I
        L.oracle_ntt.argtypes = [P, P, I, I]
        L.oracle_ntt.restype = I
        L.oracle_intt.argtypes = [P, P, I, I]
        L.oracle_intt.restype = I
        L.oracle_gl_mul.argtypes = [U64, U64]
        L.oracle_gl_mul.restype = U64
        L.oracle_gl_omega.argtypes = [I]
        L.oracle_gl_omega.restype = U64
        L.oracle_mt19937_64.argtypes = [U64, P, U64, I]
        L.oracle_mt19937_64.restype = I
        _lib = L
    return _lib


def msm(points: np.ndarray, scalars: np.ndarray, c: int = 0, threads: int = 0) -> np.ndarray:
    """One MSM: points (n, 104) uint8, scalars (n, 4) uint64 -> (144,) uint8 g1_projective_t."""
    pts = np.ascontiguousarray(points, dtype=np.uint8).reshape(-1, 104)
    sc = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    assert pts.shape[0] == sc.shape[0]
    out = np.zeros(144, dtype=np.uint8)
    lib().oracle_msm(pts.ctypes.data, sc.ctypes.data, pts.shape[0], c, threads, out.ctypes.data)
    return out


def gen_bases(seed: int, n: int, first: int = 0, threads: int = 0) -> np.ndarray:
    out = np.zeros((n, 104), dtype=np.uint8)
    lib().oracle_gen_bases(seed, first, n, out.ctypes.data, threads)
    return out


def gen_scalars(seed: int, n: int, kind: int = 0, msm_index: int = 0, threads: int = 0) -> np.ndarray:
    """Seeded scalars as (n, 4) uint64: kind 0 uniform in [0, r), kind 1 the uneven-batch mix of
    MSM `msm_index` (the draws of oracle/bls12_377.py uniform_scalar / mixed_scalar)."""
    out = np.zeros((n, 4), dtype=np.uint64)
    if lib().oracle_gen_scalars(seed, n, kind, msm_index, out.ctypes.data, threads) != 0:
        raise ValueError(f"unknown scalar kind {kind}")
    return out


def mul(point: np.ndarray, k: int) -> np.ndarray:
    p = np.ascontiguousarray(point, dtype=np.uint8).reshape(104)
    kk = np.array([(k >> (64 * i)) & (2**64 - 1) for i in range(4)], dtype=np.uint64)
    out = np.zeros(144, dtype=np.uint8)
    lib().oracle_mul(p.ctypes.data, kk.ctypes.data, out.ctypes.data)
    return out


def default_window(n: int) -> int:
    return lib().oracle_default_window(n)


# ---- NTT track (Goldilocks field) ----
GL_P = 0xFFFFFFFF00000001


def ntt(values: np.ndarray, threads: int = 0, inverse: bool = False) -> np.ndarray:
    """Forward (or inverse) NTT of 2^k Goldilocks elements, natural order in and out
    (oracle/cpu_ntt.c; the reference's host model zprize/ntt/host/reference.cpp:94-139)."""
    x = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1)
    n = x.shape[0]
    logn = n.bit_length() - 1
    if n == 0 or (1 << logn) != n:
        raise ValueError("the NTT length must be a power of two")
    out = np.empty_like(x)
    fn = lib().oracle_intt if inverse else lib().oracle_ntt
    if fn(out.ctypes.data, x.ctypes.data, logn, threads) != 0:
        raise ValueError("unsupported NTT length")
    return out


def gl_mul(a: int, b: int) -> int:
    return int(lib().oracle_gl_mul(a, b))


def gl_omega(i: int) -> int:
    return int(lib().oracle_gl_omega(i))


def mt19937_64(n: int, seed: int = 5489, mod_p: bool = True) -> np.ndarray:
    """n draws of MT19937-64 (std::mt19937_64; 5489 is its default seed), taken modulo p as the
    reference host's NTT test does (zprize/ntt/host/test_random.cpp)."""
    out = np.empty(n, dtype=np.uint64)
    lib().oracle_mt19937_64(seed, out.ctypes.data, n, 1 if mod_p else 0)
    return out
