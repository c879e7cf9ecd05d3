"""hdog_ccl_noalloc: labelling for callers that may not allocate device memory.

Such callers (a host framework that owns every device allocation through its own
allocator, or a service whose memory budget is reserved at start-up) pass the mask and
the label array; the library keeps the labelling's scratch in one fixed device array.
The labels are checked against the CPU oracle and against the context-based hdog_ccl.
This file is collected last so that a failure here comes after every other test ran.
"""
import ctypes

import numpy as np
import pytest

import hdog
from helpers import params, volume
from oracle import oracle as orc

MAX_VOXELS = 1 << 22


def test_noalloc_rejects_volumes_beyond_its_scratch():
    # checked before any device work, so this runs without a GPU
    for W, H, D in ((512, 512, 32), (256, 256, 65), (257, 256, 64)):
        assert W * H * D > MAX_VOXELS
        rc = hdog.lib().hdog_ccl_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), W, H, D, None)
        assert rc == hdog.HDOG_ERR_SHAPE
        assert b"2^22" in hdog.lib().hdog_last_error()


def _noalloc(mask, W, H, D):
    import torch
    out = torch.full((D, H, W), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = hdog.lib().hdog_ccl_noalloc(ctypes.c_void_p(mask.data_ptr()), ctypes.c_void_p(out.data_ptr()), W, H, D,
                                     ctypes.c_void_p(stream))
    assert rc == hdog.HDOG_OK, hdog.lib().hdog_last_error()
    return out.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_labels_equal_oracle_and_context_labels_on_consecutive_calls():
    import torch
    W, H, D = 200, 150, 40          # 1.2 M voxels; W not a multiple of 16
    vol = volume(W, H, D, n_nuclei=120, seed=31)
    p = params(W, H, D)
    with hdog.Context(p) as ctx:
        img = torch.from_numpy(vol).cuda()
        mask, _ = ctx.hessian_pd(ctx.dog(ctx.normalize(img)))
        ctx_labels = ctx.ccl(mask).cpu().numpy()
    ref, _ = orc.ccl(mask.cpu().numpy())
    assert np.array_equal(ctx_labels, ref)
    assert int((ref > 0).sum()) > 1000
    # a second, different mask: the shared scratch must not carry state between calls
    rng = np.random.default_rng(5)
    m2 = (rng.random((D, H, W)) < 0.3).astype(np.uint8)
    ref2, _ = orc.ccl(m2)
    mask2 = torch.from_numpy(m2).cuda()
    for m, r in ((mask, ref), (mask2, ref2), (mask, ref)):
        assert np.array_equal(_noalloc(m, W, H, D), r)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["dense_random", "sparse_random"])
def test_noalloc_at_its_voxel_limit(kind):
    """Exactly 2^22 voxels (256 x 256 x 64: 16-byte rows, row and slice wrap-around edges),
    a dense and a sparse random mask, two calls each."""
    import torch
    W, H, D = 256, 256, 64
    assert W * H * D == MAX_VOXELS
    rng = np.random.default_rng(17 if kind == "dense_random" else 18)
    m = (rng.random((D, H, W)) < (0.5 if kind == "dense_random" else 0.08)).astype(np.uint8)
    ref, _ = orc.ccl(m)
    mask = torch.from_numpy(m).cuda()
    for _ in range(2):
        assert np.array_equal(_noalloc(mask, W, H, D), ref)
