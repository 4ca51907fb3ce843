"""Readers and writers for the reference harness's test-data files.

`TEST_WRITE_DATA_TO` / `TEST_LOAD_DATA_FROM` (zprize/msm_pippenger/test_fpga_harness/src/
util.rs:126-172) store three files written with ark-serialize 0.3 `serialize_unchecked`:

    points.bin            Vec<G1Affine>   u64 count, then per point x (48 B), y (48 B), infinity (1 B)
    scalars.bin           Vec<Fr>         u64 count, then 32 B per scalar
    arkworks_results.bin  Vec<G1Affine>   the expected MSM results, one per batch

Field elements in the files are canonical little-endian integers.  The C ABI carries arkworks'
in-memory Montgomery form: coordinates as x * 2^384 mod q, and scalars as the raw Montgomery
integer of Fr (v * 2^256 mod r), which the harness transmutes into BigInteger256 before calling
msm_mult (tests/msm.rs:30-32).  The conversions run in libdriver.so on all host cores.

The layout follows ark-serialize 0.3.0's published unchecked encoding; the crate source is not
part of the reference tree.
"""
from __future__ import annotations

import os
from typing import List, Tuple

import numpy as np

from . import AFFINE_BYTES, PROJ_BYTES, MsmError, load_library

POINT_RECORD = 97  # x, y, infinity


def _check(rc: int, what: str):
    if rc != 0:
        raise MsmError(f"{what}: an element is not below the modulus")


def _read_vec(path: str, record: int) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size < 8:
        raise MsmError(f"{path}: shorter than a length prefix")
    n = int(raw[:8].view(np.uint64)[0])
    if raw.size != 8 + n * record:
        raise MsmError(f"{path}: {raw.size} bytes for {n} records of {record} bytes")
    return raw[8:].reshape(n, record)


def _write_vec(path: str, recs: np.ndarray):
    with open(path, "wb") as f:
        f.write(np.array([recs.shape[0]], dtype=np.uint64).tobytes())
        f.write(np.ascontiguousarray(recs, dtype=np.uint8).tobytes())


def read_points(path: str) -> np.ndarray:
    """points.bin -> (n, 104) g1_affine_t records in Montgomery form."""
    rec = _read_vec(path, POINT_RECORD)
    n = rec.shape[0]
    xy = np.ascontiguousarray(rec[:, :96]).view(np.uint64).reshape(n, 12).copy()
    inf = rec[:, 96] != 0
    lib = load_library()
    _check(lib.msm_fq_to_montgomery(xy.ctypes.data, 2 * n), "points")
    out = np.zeros((n, AFFINE_BYTES), dtype=np.uint8)
    out[:, :96] = xy.view(np.uint8).reshape(n, 96)
    out[:, 96] = inf
    # arkworks' zero() is (0, 1, true); the ABI only reads the flag, keep the coordinates as read
    return out


def write_points(path: str, points: np.ndarray):
    """(n, 104) g1_affine_t records (Montgomery form) -> points.bin."""
    pts = np.ascontiguousarray(points, dtype=np.uint8).reshape(-1, AFFINE_BYTES)
    n = pts.shape[0]
    xy = np.ascontiguousarray(pts[:, :96]).view(np.uint64).reshape(n, 12).copy()
    _check(load_library().msm_fq_from_montgomery(xy.ctypes.data, 2 * n), "points")
    rec = np.zeros((n, POINT_RECORD), dtype=np.uint8)
    rec[:, :96] = xy.view(np.uint8).reshape(n, 96)
    rec[:, 96] = pts[:, 96] != 0
    _write_vec(path, rec)


def read_scalars(path: str) -> np.ndarray:
    """scalars.bin -> (n, 4) u64: the raw integers the harness passes to msm_mult."""
    rec = _read_vec(path, 32)
    v = np.ascontiguousarray(rec).view(np.uint64).reshape(-1, 4).copy()
    _check(load_library().msm_fr_to_montgomery(v.ctypes.data, v.shape[0]), "scalars")
    return v


def write_scalars(path: str, scalars: np.ndarray):
    """(n, 4) raw Montgomery-form scalar integers (each < r) -> scalars.bin (canonical Fr)."""
    v = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4).copy()
    _check(load_library().msm_fr_from_montgomery(v.ctypes.data, v.shape[0]), "scalars")
    _write_vec(path, v.view(np.uint8).reshape(-1, 32))


def projective_to_affine_records(results: np.ndarray) -> np.ndarray:
    """g1_projective_t results of msm_mult (Z = R or 0) -> g1_affine_t records."""
    res = np.ascontiguousarray(results, dtype=np.uint8).reshape(-1, PROJ_BYTES)
    out = np.zeros((res.shape[0], AFFINE_BYTES), dtype=np.uint8)
    for i, p in enumerate(res):
        if not p[96:144].any():
            out[i, 96] = 1
        else:
            out[i, :96] = p[:96]
    return out


def load_test_data(directory: str) -> Tuple[int, np.ndarray, np.ndarray, np.ndarray]:
    """The TEST_LOAD_DATA_FROM branch of generate_or_load_test_data (util.rs:236-257):
    (batches, points, scalars, expected affine results)."""
    pts = read_points(os.path.join(directory, "points.bin"))
    sc = read_scalars(os.path.join(directory, "scalars.bin"))
    res = read_points(os.path.join(directory, "arkworks_results.bin"))
    if pts.shape[0] == 0 or sc.shape[0] % pts.shape[0] or sc.shape[0] < pts.shape[0]:
        raise MsmError("scalar count is not a positive multiple of the point count")
    return sc.shape[0] // pts.shape[0], pts, sc, res


def save_test_data(directory: str, points: np.ndarray, scalars: np.ndarray, results: np.ndarray):
    """The TEST_WRITE_DATA_TO branch (util.rs:211-232)."""
    os.makedirs(directory, exist_ok=True)
    write_points(os.path.join(directory, "points.bin"), points)
    write_scalars(os.path.join(directory, "scalars.bin"), scalars)
    write_points(os.path.join(directory, "arkworks_results.bin"), projective_to_affine_records(results))
