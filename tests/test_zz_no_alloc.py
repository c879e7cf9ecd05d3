"""hdog_ccl_noalloc: labelling for callers that may not allocate device memory.

Such callers (a host framework that owns every device allocation through its own
allocator, or a service whose memory budget is reserved at start-up) pass the mask and
the label array; the library keeps the labelling's scratch in one fixed device array.
This file is collected last so that a failure here comes after every other test ran.
"""
import ctypes

import numpy as np
import pytest

import hdog
from helpers import params, volume


def test_noalloc_rejects_volumes_beyond_its_scratch():
    # checked before any device work, so this runs without a GPU
    rc = hdog.lib().hdog_ccl_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 512, 512, 32, None)
    assert rc == hdog.HDOG_ERR_SHAPE
    assert b"2^22" in hdog.lib().hdog_last_error()


@pytest.mark.gpu
def test_noalloc_labels_equal_context_labels_on_consecutive_calls():
    import torch
    W, H, D = 200, 150, 40          # 1.2 M voxels, under the 2^22 limit
    vol = volume(W, H, D, n_nuclei=120, seed=31)
    p = params(W, H, D)
    with hdog.Context(p) as ctx:
        img = torch.from_numpy(vol).cuda()
        mask, _ = ctx.hessian_pd(ctx.dog(ctx.normalize(img)))
        ref = ctx.ccl(mask).cpu().numpy()
    # a second, different mask: the shared scratch must not carry state between calls
    rng = np.random.default_rng(5)
    mask2 = torch.from_numpy((rng.random((D, H, W)) < 0.3).astype(np.uint8)).cuda()
    with hdog.Context(p) as ctx:
        ref2 = ctx.ccl(mask2).cpu().numpy()
    stream = torch.cuda.current_stream().cuda_stream
    for m, r in ((mask, ref), (mask2, ref2), (mask, ref)):
        out = torch.full((D, H, W), -7, dtype=torch.int32, device="cuda")
        rc = hdog.lib().hdog_ccl_noalloc(ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(out.data_ptr()), W, H, D,
                                         ctypes.c_void_p(stream))
        assert rc == hdog.HDOG_OK, hdog.lib().hdog_last_error()
        assert np.array_equal(out.cpu().numpy(), r)
    assert int((ref > 0).sum()) > 1000
