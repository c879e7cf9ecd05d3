"""The CPU oracle checked against independent numpy / scipy restatements.

Exactness notes: min/max, box sums, gradients and the no-contraction Sylvester test are
compared bit for bit (numpy float32 performs the same IEEE operations in the same
order); the FMA-chain Gaussian is compared against float64 within 1e-5 (numpy has no
fused multiply-add); the pinning of the FMA forms against the reference's own kernels
is in test_cpu_golden.py.
"""
import numpy as np
import pytest
import scipy.ndimage as ndi

from oracle import oracle as orc
from helpers import volume, rel_close


def rng_vol(shape, seed, lo=0, hi=4000):
    return np.random.default_rng(seed).integers(lo, hi, size=shape, dtype=np.uint16)


@pytest.mark.parametrize("shape,rxy,rz", [((7, 13, 17), 2, 1), ((16, 20, 24), 5, 3), ((5, 9, 11), 12, 6)])
def test_minmax_nearest_matches_scipy(shape, rxy, rz):
    v = rng_vol(shape, 1)
    ero, dil = orc.minmax3d(v, rxy, rz)
    size = (2 * rz + 1, 2 * rxy + 1, 2 * rxy + 1)
    assert np.array_equal(ero, ndi.minimum_filter(v, size=size, mode="nearest"))
    assert np.array_equal(dil, ndi.maximum_filter(v, size=size, mode="nearest"))


def np_box_nearest(a, r, axis):
    """Sequential float32 window sum from 0.0f in tap order, nearest border, then * 1/(2r+1)."""
    a = a.astype(np.float32)
    n = a.shape[axis]
    acc = np.zeros_like(a)
    for j in range(2 * r + 1):
        idx = np.clip(np.arange(n) - r + j, 0, n - 1)
        acc = (acc + np.take(a, idx, axis=axis)).astype(np.float32)
    return (acc * (np.float32(1.0) / np.float32(2 * r + 1))).astype(np.float32)


@pytest.mark.parametrize("shape,rxy,rz", [((8, 12, 20), 3, 2), ((6, 31, 9), 7, 4)])
def test_normalize_bit_exact_vs_numpy(shape, rxy, rz):
    v = rng_vol(shape, 2, 50, 3000)
    norm, ero_l, dil_l = orc.normalize(v, rxy, rz, 100.0, want_parts=True)
    size = (2 * rz + 1, 2 * rxy + 1, 2 * rxy + 1)
    e = ndi.minimum_filter(v, size=size, mode="nearest")
    d = ndi.maximum_filter(v, size=size, mode="nearest")

    def box(m):
        b = np_box_nearest(m, rxy, 2)
        b = np_box_nearest(b, rxy, 1)
        return np_box_nearest(b, rz, 0)

    E, Dl = box(e), box(d)
    assert np.array_equal(ero_l.view(np.uint32), E.view(np.uint32))
    assert np.array_equal(dil_l.view(np.uint32), Dl.view(np.uint32))
    I = v.astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = np.where(I >= np.float32(100.0), ((I - E) / (Dl - E)).astype(np.float32), np.float32(0))
    assert np.array_equal(norm.view(np.uint32), ref.astype(np.float32).view(np.uint32))


def test_normalize_radius_zero_is_copy():
    v = rng_vol((4, 5, 6), 3)
    n = orc.normalize(v, 0, 3, 1000.0)
    assert np.array_equal(n, np.where(v >= 1000, v, 0).astype(np.float32))


def test_gauss3d_close_to_float64():
    v = np.random.default_rng(4).random((11, 17, 23)).astype(np.float32)
    out = orc.gauss3d(v, 2.0, 1.5)
    kxy, rxy = orc.gauss_taps(2.0)
    kz, rz = orc.gauss_taps(1.5)
    a = v.astype(np.float64)
    for axis, k, r in ((2, kxy, rxy), (1, kxy, rxy), (0, kz, rz)):
        a = ndi.correlate1d(a, k[: 2 * r + 1].astype(np.float64), axis=axis, mode="constant", cval=0.0)
    assert rel_close(out, a, 1e-5, 1e-7)


def np_grad(f, axis):
    n = f.shape[axis]
    pad = [(0, 0)] * 3
    pad[axis] = (1, 1)
    g = np.pad(f, pad)
    plus = np.take(g, np.arange(2, n + 2), axis=axis)
    minus = np.take(g, np.arange(0, n), axis=axis)
    return (((np.float32(0) + plus).astype(np.float32) - minus).astype(np.float32) * np.float32(0.5)).astype(np.float32)


def test_hessian_planes_and_plain_pd_bit_exact():
    rng = np.random.default_rng(5)
    dog = (rng.standard_normal((9, 14, 19)) * 0.1).astype(np.float32)
    mask, hess = orc.hessian_pd(dog, pd_variant=0, want_hessian=True)
    gx, gy, gz = np_grad(dog, 2), np_grad(dog, 1), np_grad(dog, 0)
    ref = [np_grad(gx, 2), np_grad(gx, 1), np_grad(gx, 0), np_grad(gy, 1), np_grad(gy, 0), np_grad(gz, 0)]
    for k in range(6):
        assert np.array_equal(hess[k].view(np.uint32), ref[k].view(np.uint32)), k
    xx, xy, xz, yy, yz, zz = ref
    f = np.float32
    m2 = (xx * yy).astype(f) - (xy * xy).astype(f)
    det = ((((((xx * yy).astype(f) * zz).astype(f) + (((f(2) * xy).astype(f) * yz).astype(f) * xz).astype(f))
             - ((xx * yz).astype(f) * yz).astype(f)) - ((yy * xz).astype(f) * xz).astype(f))
           - ((zz * xy).astype(f) * xy).astype(f))
    pd = (xx < 0) & (m2 > 0) & (det < 0)
    assert np.array_equal(mask.astype(bool), pd)
    assert pd.sum() > 0


def test_hessian_at_matches_planes():
    dog = (np.random.default_rng(6).standard_normal((6, 7, 8))).astype(np.float32)
    _, hess = orc.hessian_pd(dog, want_hessian=True)
    # the per-voxel recomputation used for region sums equals the plane pass
    r = orc.regions(np.where(np.ones(dog.shape, bool), 1, 0).astype(np.int32) * 0, np.zeros_like(dog), dog)
    assert r["num_regions"] == 1
    lab = np.zeros(dog.shape, np.int32)
    lab.flat[1:] = 1
    lab.flat[1] = 1
    r = orc.regions(lab, np.zeros_like(dog), dog)
    s64 = hess.reshape(6, -1)[:, 1:].astype(np.float64).sum(axis=1)
    assert rel_close(r["hess_f64"][:, 1], s64, 1e-12, 1e-12)


def ccl_by_scipy(mask):
    lab, n = ndi.label(mask, structure=np.ones((3, 3, 3), int))
    out = np.zeros(mask.shape, np.int32)
    flat = lab.ravel()
    idx = np.arange(flat.size)
    mins = np.full(n + 1, np.iinfo(np.int64).max)
    np.minimum.at(mins, flat, idx)
    out.ravel()[:] = np.where(flat > 0, mins[flat], 0)
    return out, n + 1


def test_ccl_interior_matches_scipy_min_index_labels():
    rng = np.random.default_rng(7)
    m = (rng.random((10, 20, 30)) < 0.2).astype(np.uint8)
    m[:, :, 0] = 0
    m[:, :, -1] = 0      # no wrap from a row end to the next row's start (offset +-1)
    m[:, 0, :] = 0
    m[:, -1, :] = 0      # no wrap from a slice's last row to the next slice's first (offset +-W)
    lab, n = orc.ccl(m)
    ref, nref = ccl_by_scipy(m)
    assert n == nref
    assert np.array_equal(lab, ref)


def test_ccl_wraps_linear_offsets_and_drops_voxel_zero():
    D, H, W = 4, 5, 6
    m = np.zeros((D, H, W), np.uint8)
    m[1, 2, W - 1] = 1       # row end ...
    m[1, 3, 0] = 1           # ... touches the next row's start (offset +1)
    m[2, H - 1, 3] = 1       # last row of slice 2 ...
    m[3, 0, 3] = 1           # ... touches the first row of slice 3 (offset +W)
    m[0, 0, 0] = 1           # voxel 0 is background (label = index * mask)
    m[0, 0, 1] = 1
    lab, n = orc.ccl(m)
    i = lambda z, y, x: (z * H + y) * W + x
    assert lab[1, 2, W - 1] == lab[1, 3, 0] == i(1, 2, W - 1)
    assert lab[2, H - 1, 3] == lab[3, 0, 3] == i(2, H - 1, 3)
    assert lab[0, 0, 0] == 0 and lab[0, 0, 1] == 1
    assert n == 4


def test_ccl_on_filled_volume_is_one_region():
    m = np.ones((3, 4, 5), np.uint8)
    lab, n = orc.ccl(m)
    assert n == 2 and lab.flat[0] == 0 and np.all(lab.flat[1:] == 1)


def test_regions_counts_max_centroids():
    rng = np.random.default_rng(8)
    m = (rng.random((6, 15, 17)) < 0.3).astype(np.uint8)
    lab, n = orc.ccl(m)
    norm = rng.random(m.shape).astype(np.float32)
    dog = rng.standard_normal(m.shape).astype(np.float32)
    r = orc.regions(lab, norm, dog)
    assert r["num_regions"] == n
    roots = np.sort(np.unique(lab[lab > 0]))
    assert np.array_equal(r["label"][1:], roots)
    for k, L in enumerate(roots[:20], start=1):
        sel = lab == L
        assert r["count"][k] == sel.sum()
        assert r["max_norm"][k] == norm[sel].max()
        z, y, x = np.nonzero(sel)
        assert r["sum_xyz"][0, k] == x.sum() and r["sum_xyz"][1, k] == y.sum() and r["sum_xyz"][2, k] == z.sum()


def test_eigen_matches_numpy():
    rng = np.random.default_rng(9)
    for _ in range(200):
        a = rng.standard_normal((3, 3))
        s = (a + a.T).astype(np.float32)
        hs = np.array([s[0, 0], s[0, 1], s[0, 2], s[1, 1], s[1, 2], s[2, 2]], np.float32)
        st, bl = orc.eigen(hs)
        ev = np.linalg.eigvalsh(s.astype(np.float64))
        assert abs(st - (ev ** 2).sum()) <= 1e-5 * max(1.0, (ev ** 2).sum())
        ref_bl = ev[2] ** 2 / (ev[0] * ev[1])
        assert abs(bl - ref_bl) <= 1e-4 * max(1.0, abs(ref_bl))
    # diagonal input keeps the unsorted diagonal (Eigenvalues.cu:81-85)
    st, bl = orc.eigen(np.array([-3, 0, 0, -1, 0, -2], np.float32))
    assert st == 14.0 and bl == np.float32(4.0 / 3.0)
    assert orc.eigen(np.zeros(6, np.float32)) == (0.0, 0.0)


@pytest.mark.parametrize("rxy,rz", [(1, 1), (2, 0), (3, 2)])
def test_erosion_zero_border_matches_scipy(rxy, rz):
    v = rng_vol((9, 11, 13), 10, 1, 60000)
    out = orc.erosion(v, rxy, rz)
    ref = ndi.minimum_filter(v, size=(2 * rz + 1, 2 * rxy + 1, 2 * rxy + 1), mode="constant", cval=0)
    assert np.array_equal(out, ref)


def test_substack_records_are_sane():
    import hdog
    v = volume(256, 256, 32, n_nuclei=200)
    p = hdog.make_params(width=256, height=256, depth=32, sigma_xy_small=2.0, sigma_z_small=1.5,
                         sigma_xy_large=3.2, sigma_z_large=2.4, radius_norm_xy=20, radius_norm_z=5,
                         min_intensity=50, min_size=0, left_margin=0, right_margin=0, top_margin=0, bottom_margin=0)
    op = orc.params_from(p)
    recs, nreg, mask, labels = orc.substack(op, v, 32, 100)
    assert nreg > 50 and len(recs) > 20
    m = orc.depth_margin(op)
    assert np.all(recs["local_z"] >= 100 + m) and np.all(recs["local_z"] < 100 + 32 - m)
    assert np.all(recs["intensity"] > 0) and np.all(recs["padding"] == 0)
    # records come in region order = ascending label; labels of kept regions are roots
    roots = np.unique(labels[labels > 0])
    assert nreg == len(roots) + 1
