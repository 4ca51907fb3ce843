"""The entry point that allocates no device memory (msm_mult_noalloc).

It serves callers that cannot allocate device memory at call time, such as a plugin inside
another runtime's memory pool or a request loop that must not stall on cudaMalloc.  The test
allocates the scalars and the output itself, calls the entry point twice in a row through the
C ABI, and requires each result to equal the existing entry point's result byte for byte.  This
file runs last so that a failure here cannot hide other failures.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_existing_entry_point_twice(engine, ocpu):
    import torch

    nbase = 6000
    pts = ocpu.gen_bases(909, nbase)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        for call, (n, off) in enumerate(((5000, 1000), (4096, 0))):
            sc = engine.generate_scalars(910 + call, n)
            d_sc = torch.from_numpy(sc.view(np.uint8).reshape(-1)).cuda()
            d_out = torch.zeros(144, dtype=torch.uint8, device="cuda")
            torch.cuda.synchronize()
            ctx.mult_noalloc(n, off, d_sc.data_ptr(), d_out.data_ptr())
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            want = ctx.mult_uneven([n], [off], sc)[0]
            assert np.array_equal(got, want), f"call {call}"
            assert np.array_equal(got, ocpu.msm(pts[off:off + n], sc))
    finally:
        ctx.close()


def test_noalloc_at_the_maximum_size_and_empty(engine, ocpu):
    """n = 65536 (the largest size the array holds; the only caller of the unstaged scatter at
    that size) against the existing entry point and the oracle, then n = 0, which must give
    arkworks' zero (R, R, 0)."""
    import torch

    nbase = 70000
    pts = ocpu.gen_bases(911, nbase)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        n, off = 1 << 16, 4000
        sc = engine.generate_scalars(912, n)
        d_sc = torch.from_numpy(sc.view(np.uint8).reshape(-1)).cuda()
        d_out = torch.zeros(144, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        ctx.mult_noalloc(n, off, d_sc.data_ptr(), d_out.data_ptr())
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.array_equal(got, ctx.mult_uneven([n], [off], sc)[0])
        assert np.array_equal(got, ocpu.msm(pts[off:off + n], sc))
        d_out.fill_(0xAB)
        ctx.mult_noalloc(0, 0, d_sc.data_ptr(), d_out.data_ptr())
        torch.cuda.synchronize()
        zero = ocpu.msm(pts[:0], sc[:0])
        assert np.array_equal(d_out.cpu().numpy(), zero)
    finally:
        ctx.close()


def test_noalloc_rejects_sizes_over_the_maximum(engine, ocpu):
    import torch

    pts = ocpu.gen_bases(5, 70000)
    ctx = engine.multi_scalar_mult_init(pts)
    try:
        d_sc = torch.zeros(70000 * 32, dtype=torch.uint8, device="cuda")
        d_out = torch.zeros(144, dtype=torch.uint8, device="cuda")
        with pytest.raises(engine.MsmError, match="maximum of 65536"):
            ctx.mult_noalloc(65537, 0, d_sc.data_ptr(), d_out.data_ptr())
    finally:
        ctx.close()
