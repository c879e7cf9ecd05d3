"""Records against the reference's own code path (oracle/ref_records.py): the reference's
stage kernels compiled unmodified, its CUB region reductions restated call for call, its
record filter.  Needs the reference's kernels as cubins (built where the reference checkout
is present, oracle/build_oracle.py); skipped without them.

On a 1280 x 2160 x 48 stack (two substacks of depth 32, inside the reference kernels'
launch geometry): record count and order, centroids, size and intensity bit for bit;
structureness and blobness within EIGEN_RTOL of the reference path's; the region Hessian
sums of substack 0 within SUM_RTOL of the region's largest element of the reference's CUB
sums; and both paths' eigen features against FP64.
"""
import numpy as np
import pytest
import torch

import hdog
from helpers import params, volume
from oracle import oracle as orc
from oracle import ref_cubin

pytestmark = pytest.mark.gpu

EXACT = ("local_x", "local_y", "local_z", "intensity", "size", "padding")
# Float sums: the reference's CUB reduce-by-key in float32 against this library's 2^-36
# fixed point.  The eigen features amplify their difference where eigenvalues nearly
# cancel; on this stack they stay within 1e-5 relative of the reference path's (measured:
# structureness 4.6e-7, blobness 3.0e-6), the bound the float features are held to.
SUM_RTOL = 1e-5
EIGEN_RTOL = 1e-5


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-30)


@pytest.fixture(scope="module")
def case():
    if not ref_cubin.available():
        pytest.skip("the reference's kernels were not built (no reference checkout where this was built)")
    from oracle import ref_records
    W, H, L = 1280, 2160, 48
    p = params(W, H, 32, margins=20)
    vol = volume(W, H, L, n_nuclei=int(W * H * L / 11800), seed=4242, pair_fraction=0.1)
    dev = torch.from_numpy(vol).cuda()
    op = orc.params_from(p)
    margin = orc.depth_margin(op)
    sched = orc.schedule(L, p.depth, margin)
    normalizer = orc.dog_normalizer(p.sigma_xy_small, p.sigma_z_small, p.gamma_n)
    ref, st64, bl64 = ref_records.stack(dev, p, orc.gauss_taps, normalizer, margin, sched)
    with hdog.Context(p, max_substacks=len(sched)) as ctx:
        ours = ctx.run_stack(dev)
    sub0 = dev[:p.depth].contiguous()
    rec0, _, vols = ref_records.substack(sub0, p.depth, 0, p, orc.gauss_taps, normalizer, margin)
    return dict(p=p, ref=ref, ours=ours, st64=st64, bl64=bl64, vols=vols, ref_records=ref_records)


def test_exact_record_fields_equal_the_reference_path(case):
    ref, ours = case["ref"], case["ours"]
    assert len(ref) > 1000
    assert len(ours) == len(ref)
    for f in EXACT:
        assert np.array_equal(ours[f], ref[f]), f


def test_eigen_features_and_their_fp64_error(case):
    ref, ours = case["ref"], case["ours"]
    for f, f64 in (("structureness", case["st64"]), ("blobness", case["bl64"])):
        d = _rel(ours[f], ref[f])
        e_ours = _rel(ours[f], f64)
        e_ref = _rel(ref[f], f64)
        print("%s: max rel vs reference %.3g; vs FP64: ours %.3g, reference %.3g (99.9th pct %.3g / %.3g)"
              % (f, d.max(), e_ours.max(), e_ref.max(), np.quantile(e_ours, 0.999), np.quantile(e_ref, 0.999)))
        assert d.max() <= EIGEN_RTOL, f
        # the fixed-point sums are at least as close to the exact sums as the float ones
        assert np.quantile(e_ours, 0.999) <= np.quantile(e_ref, 0.999) * 1.01 + 1e-7, f


def test_region_hessian_sums_against_the_reference_cub_sums(case):
    v = case["vols"]
    p = case["p"]
    with hdog.Context(p) as ctx:
        r = ctx.regional_features(v["labels"], v["norm"], v["dog"])
    hess, _ = ref_cubin.hessian_pd(v["dog"])
    f = case["ref_records"].regional_features(v["labels"], hess, v["norm"], p.is_ave_mode)
    assert r["num_regions"] == f["num_regions"]
    assert np.array_equal(r["label"], f["label"])
    # region 0 is the background (label 0), which no record reports: compare regions 1..
    fg = slice(1, None)
    assert np.array_equal((r["count"][fg] & 0xFFFF).astype(np.uint16), f["size"][fg])
    assert np.array_equal(r["intensity"][fg].view(np.uint32), f["intensity"][fg].view(np.uint32))
    # centroids: coordinate sums are exact in float only below 2^24, so compare the regions
    # whose sums stay below it (larger ones follow CUB's float association)
    small = (r["count"][fg].astype(np.float64) * np.array([p.width, p.height, p.depth])[:, None] < 2 ** 24).all(0)
    assert small.mean() > 0.99
    assert np.array_equal(r["centroid"][:, fg][:, small].view(np.uint32), f["centroid"][:, fg][:, small].view(np.uint32))
    scale = np.maximum(np.abs(f["hessian"][:, fg]).max(axis=0), 1e-30)
    err = np.abs(r["hessian"][:, fg].astype(np.float64) - f["hessian"][:, fg]) / scale
    print("region Hessian sums: max |ours - reference| / region scale = %.3g" % err.max())
    assert err.max() <= SUM_RTOL
