"""Multi-GPU form of one MSM: split the bases into contiguous slices, one per rank.

An MSM is a sum of independent partial MSMs, so rank r computes the partial sum over its slice
of (scalar, base) pairs on its own GPU.  The one exchange is a gather of one 144-byte
g1_projective_t per rank, plus one status word, over torch.distributed (gloo or NCCL).  Every
rank then adds the partial points.  The reference has no multi-device path; this is the sharding
its single FPGA did not need.

A rank whose partial computation raises still joins the gather, carrying a failure status, so
the other ranks raise instead of waiting.  A rank that dies outright surfaces through the process
group's own timeout.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

import numpy as np

PROJ_BYTES = 144


def partition(n: int, world: int) -> List[Tuple[int, int]]:
    """Balanced contiguous slices [lo, hi) of n items over `world` ranks."""
    if world <= 0:
        raise ValueError("world size must be positive")
    base, extra = divmod(n, world)
    out, lo = [], 0
    for r in range(world):
        hi = lo + base + (1 if r < extra else 0)
        out.append((lo, hi))
        lo = hi
    return out


class ShardError(RuntimeError):
    pass


def gather_partials(part: np.ndarray, ok: bool, group=None) -> List[np.ndarray]:
    """All-gather one 144-byte result and a status byte from every rank."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rec = np.zeros(PROJ_BYTES + 8, dtype=np.uint8)
    rec[:PROJ_BYTES] = part if ok else 0
    rec[PROJ_BYTES] = 1 if ok else 0
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.from_numpy(rec.copy()).to(dev)
    outs = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(outs, t, group=group)
    recs = [o.cpu().numpy() for o in outs]
    bad = [r for r, x in enumerate(recs) if x[PROJ_BYTES] != 1]
    if bad:
        raise ShardError(f"partial MSM failed on rank(s) {bad}")
    return [x[:PROJ_BYTES].copy() for x in recs]


def sharded_msm(n: int, rank: int, world: int,
                partial_fn: Callable[[int, int], np.ndarray],
                combine_fn: Callable[[Sequence[np.ndarray]], np.ndarray],
                group=None) -> np.ndarray:
    """Run this rank's share of one MSM and return the full result on every rank.

    partial_fn(lo, hi) returns the g1_projective_t of sum_{lo <= i < hi} k_i P_i.
    combine_fn(parts) adds the per-rank points (in rank order).
    """
    lo, hi = partition(n, world)[rank]
    try:
        part = np.asarray(partial_fn(lo, hi), dtype=np.uint8).reshape(PROJ_BYTES)
        ok = True
    except Exception:
        part = np.zeros(PROJ_BYTES, dtype=np.uint8)
        ok = False
    parts = gather_partials(part, ok, group)
    if not ok:
        raise ShardError(f"partial MSM failed on rank {rank}")
    return combine_fn(parts)


def projective_to_affine_records(parts: Sequence[np.ndarray]) -> np.ndarray:
    """g1_projective_t results (Z = R or 0) -> g1_affine_t records for a combining MSM."""
    out = np.zeros((len(parts), 104), dtype=np.uint8)
    for i, p in enumerate(parts):
        p = np.asarray(p, dtype=np.uint8)
        z = p[96:144]
        if not z.any():
            out[i, 48:96] = p[48:96]
            out[i, 96] = 1
        else:
            out[i, :96] = p[:96]
    return out


def combine_on_gpu(parts: Sequence[np.ndarray]) -> np.ndarray:
    """Add the partial points with the engine itself: an MSM of the partials with scalars 1."""
    from . import multi_scalar_mult, multi_scalar_mult_init

    pts = projective_to_affine_records(parts)
    ctx = multi_scalar_mult_init(pts)
    try:
        ones = np.zeros((len(parts), 4), dtype=np.uint64)
        ones[:, 0] = 1
        return multi_scalar_mult(ctx, pts, ones)[0]
    finally:
        ctx.close()
