"""Stage-wise parity of the sm_103a kernels with the CPU oracle, through the C ABI.

Bit-exact: normalized volume, DoG, the six Hessian planes, the PD mask, CCL labels,
region counts / labels / max intensity / centroids, erosion.  Region Hessian sums are
accumulated in double on the GPU and compared with the oracle's double sums within
a relative 1e-6 of the region's scale.
"""
import numpy as np
import pytest
import torch

import hdog
from helpers import params, volume, rel_close
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

CASES = {
    "cube256x256x32": (256, 256, 32, {}),
    "odd67x45x13": (67, 45, 13, dict(radius_norm_xy=7, radius_norm_z=3)),
    "radius_wider_than_image": (96, 80, 16, dict(radius_norm_xy=100, radius_norm_z=5, sigma_xy_small=4.0,
                                                 sigma_z_small=1.8, sigma_xy_large=6.0, sigma_z_large=2.7)),
    "copy_path_r0": (64, 48, 16, dict(radius_norm_xy=0, min_intensity=120)),
    "tiny5x3x2": (5, 3, 2, dict(radius_norm_xy=2, radius_norm_z=1)),
    "wide_x_box_r140": (300, 40, 8, dict(radius_norm_xy=140, radius_norm_z=2)),
    # the radius-specialised normalize passes (r_xy 20, r_z 5) on ragged tiles and a
    # substack shallower than the z window
    "ragged_r20_203x150x19": (203, 150, 19, {}),
    "shallow_r20_64x40x6": (64, 40, 6, {}),
    # the streaming z min/max (r_z 5, W*H a multiple of 4) on 3 and 7 slices
    "shallow_r20_48x32x3": (48, 32, 3, {}),
    "odd_depth_r20_96x24x7": (96, 24, 7, {}),
}


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_bits_equal(got, ref, what):
    g, r = bits(got), bits(ref)
    bad = np.count_nonzero(g != r)
    assert bad == 0, "%s: %d of %d values differ" % (what, bad, g.size)


@pytest.fixture(scope="module", params=sorted(CASES))
def staged(request):
    W, H, D, kw = CASES[request.param]
    p = params(W, H, D, **kw)
    vol = volume(W, H, D, n_nuclei=max(3, W * H * D // 9000))
    with hdog.Context(p) as ctx:
        img = torch.from_numpy(vol).cuda()
        norm = ctx.normalize(img)
        dog = ctx.dog(norm)
        mask, hess = ctx.hessian_pd(dog, want_hessian=True)
        labels = ctx.ccl(mask)
        regs = ctx.regional_features(labels, norm, dog)
        torch.cuda.synchronize()
        gpu = dict(norm=norm.cpu().numpy(), dog=dog.cpu().numpy(), mask=mask.cpu().numpy(),
                   hess=hess.cpu().numpy(), labels=labels.cpu().numpy(), regs=regs)
    o_norm = orc.normalize(vol, p.radius_norm_xy, p.radius_norm_z, float(p.min_intensity))
    o_dog = orc.dog(o_norm, p.sigma_xy_small, p.sigma_z_small, p.sigma_xy_large, p.sigma_z_large, p.gamma_n)
    o_mask, o_hess = orc.hessian_pd(o_dog, want_hessian=True)
    o_labels, o_n = orc.ccl(o_mask)
    o_regs = orc.regions(o_labels, o_norm, o_dog)
    ref = dict(norm=o_norm, dog=o_dog, mask=o_mask, hess=o_hess, labels=o_labels, n=o_n, regs=o_regs)
    return request.param, p, vol, gpu, ref


def test_normalize(staged):
    name, p, vol, g, r = staged
    assert_bits_equal(g["norm"], r["norm"], name + " norm")


def test_dog(staged):
    name, p, vol, g, r = staged
    assert_bits_equal(g["dog"], r["dog"], name + " dog")


def test_hessian_planes_and_mask(staged):
    name, p, vol, g, r = staged
    assert_bits_equal(g["hess"], r["hess"], name + " hessian")
    assert_bits_equal(g["mask"], r["mask"], name + " pd mask")


def test_ccl_labels(staged):
    name, p, vol, g, r = staged
    assert_bits_equal(g["labels"], r["labels"], name + " labels")


def test_regional_features(staged):
    name, p, vol, g, r = staged
    G, R = g["regs"], r["regs"]
    n = R["num_regions"]
    assert G["num_regions"] == n
    assert np.array_equal(G["label"][1:], R["label"][1:])
    assert np.array_equal(G["count"][1:], R["count"][1:].astype(np.uint32))
    assert_bits_equal(G["intensity"][1:], R["max_norm"][1:], name + " max normalized intensity")
    c16 = (R["count"][1:] & 0xFFFF).astype(np.float32)
    for k in range(3):
        cent = (R["sum_xyz"][k, 1:].astype(np.float32) / c16).astype(np.float32)
        assert_bits_equal(G["centroid"][k, 1:], cent, name + " centroid %d" % k)
    scale = np.abs(R["hess_f64"][:, 1:]).max(axis=0) if n > 1 else np.zeros(0)
    for k in range(6):
        d = np.abs(G["hessian"][k, 1:].astype(np.float64) - R["hess_f64"][k, 1:])
        assert np.all(d <= 1e-6 * scale + 1e-30), (name, k, float((d / np.maximum(scale, 1e-30)).max()))


@pytest.mark.parametrize("rxy,rz", [(1, 1), (3, 2), (0, 1)])
def test_erosion_operator(rxy, rz):
    vol = volume(90, 70, 12, n_nuclei=5)
    p = params(90, 70, 12)
    with hdog.Context(p) as ctx:
        out = ctx.erosion(torch.from_numpy(vol).cuda(), rxy, rz).cpu().numpy()
    assert np.array_equal(out, orc.erosion(vol, rxy, rz))
