"""Capacity paths of the chain on the GPU, against the oracle.

- Foreground list over capacity (N/8 + 1024 entries per substack): a lattice of large bright
  spots puts about a fifth of the voxels in the negative-definite mask, so the fused sweep's
  list overflows and the batch is redone with the separate passes.  The records must equal
  the oracle's, for the radius-specialised sweep (the workload's sigmas) and for the generic
  fused kernel (other tap radii).
- Cross-tile edge list over capacity (N/8 + 1024 edges per substack): the CCL stage on a full
  mask, whose cross-tile edges exceed the list so they are merged straight from the mask, and
  on a half-density random mask that stays on the list.  The labels must equal the oracle's
  bit for bit.
"""
import numpy as np
import pytest
import torch

import hdog
from helpers import params
from oracle import oracle as orc
from test_gpu_pipeline import assert_records_match

pytestmark = pytest.mark.gpu

WORKLOAD_SIGMAS = dict(sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2, sigma_z_large=2.4)
NARROW_SIGMAS = dict(sigma_xy_small=1.0, sigma_z_small=1.0, sigma_xy_large=1.6, sigma_z_large=1.6)


def spot_lattice(W, H, D, spacing, sigma, seed=11):
    """uint16 volume: Gaussian spots of width sigma on a cubic lattice, background 100, noise 2."""
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    r2 = sum(((c % spacing) - spacing / 2.0) ** 2 for c in (x, y, z))
    rng = np.random.default_rng(seed)
    vol = 100 + 3000 * np.exp(-r2 / (2 * sigma * sigma)) + rng.normal(0, 2, r2.shape)
    return vol.clip(0, 65535).astype(np.uint16)


@pytest.mark.parametrize("spacing,sigma,dog", [(14, 5.5, WORKLOAD_SIGMAS), (8, 3.2, NARROW_SIGMAS)],
                         ids=["specialised_sweep", "generic_fused"])
def test_foreground_list_overflow_redoes_the_batch(spacing, sigma, dog):
    W, H, D = 128, 96, 32
    vol = spot_lattice(W, H, D, spacing, sigma)
    p = params(W, H, D, extra_depth_margin=0, **dog)
    # the premise: more mask voxels than the list holds
    norm = orc.normalize(vol, p.radius_norm_xy, p.radius_norm_z, float(p.min_intensity))
    dogv = orc.dog(norm, p.sigma_xy_small, p.sigma_z_small, p.sigma_xy_large, p.sigma_z_large, p.gamma_n)
    mask, _ = orc.hessian_pd(dogv, want_hessian=False)
    assert np.count_nonzero(mask) > W * H * D // 8 + 1024
    with hdog.Context(p) as ctx:
        got = ctx.run_substack(vol, D, 0)
    ref = orc.substack(orc.params_from(p), vol, D, 0)[0]
    assert len(ref) > 20
    assert_records_match(got, ref, "foreground list overflow, spacing %d" % spacing)


@pytest.mark.parametrize("kind", ["full", "random_half"])
def test_ccl_edge_list_overflow_merges_from_the_mask(kind):
    W, H, D = 256, 256, 32
    if kind == "full":
        mask = np.ones((D, H, W), np.uint8)
    else:
        mask = (np.random.default_rng(5).random((D, H, W)) < 0.5).astype(np.uint8)
    with hdog.Context(params(W, H, D)) as ctx:
        labels = ctx.ccl(torch.from_numpy(mask).cuda()).cpu().numpy()
        edges, cap = ctx.ccl_edge_count()
    # the premise: the full mask overflows the edge list, so its merges come from the mask;
    # the half-density mask stays on the list
    if kind == "full":
        assert edges > cap, (edges, cap)
    else:
        assert 0 < edges <= cap, (edges, cap)
    ref, _ = orc.ccl(mask)
    assert np.array_equal(labels, ref), kind


def test_bounded_union_find_walks_report_a_timeout_and_the_context_stays_usable():
    """A walk bound of 1 on a full mask, whose tile roots merge across many tiles: a walk
    passes the bound, the call reports HDOG_ERR_TIMEOUT (no hang), and with the default
    bound restored the same context labels the mask as the oracle does."""
    W, H, D = 256, 256, 32
    mask = torch.from_numpy(np.ones((D, H, W), np.uint8)).cuda()
    with hdog.Context(params(W, H, D)) as ctx:
        ctx.set_walk_limit(1)
        with pytest.raises(hdog.HDoGError) as e:
            ctx.ccl(mask)
        assert e.value.code == hdog.HDOG_ERR_TIMEOUT
        ctx.set_walk_limit(0)
        labels = ctx.ccl(mask).cpu().numpy()
    ref, _ = orc.ccl(np.ones((D, H, W), np.uint8))
    assert np.array_equal(labels, ref)
