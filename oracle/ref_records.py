"""TEST INFRASTRUCTURE ONLY: candidate records from the reference's own code path.

HDoG3D_main itself cannot run on the GPU hosts this project is tested on (an Arm host
without the reference checkout: its host part would have to be compiled there from the
reference's sources).  This module recomposes what it computes for each substack
(src/3D/HDoG3D_main.cpp:134-257) from pieces that do run there:
  * the reference's own stage kernels, compiled unmodified for sm_103a and launched by
    oracle/ref_cubin.py: Normalize3DFilter, DoG3DFilter, HessianPositiveDefiniteWithElement,
    CCL, EigenvaluesKernel;
  * its region reductions restated call for call with the same CUB algorithms
    (oracle/ref_features.cu: RegionalFeatures.cu:65-87,114-137,157-255,295-329);
  * its record filter and layout, saveFeatureVector (src/3D/utils.h:204-250), restated in
    numpy below, and the substack schedule of main (HDoG3D_main.cpp:279-315).
It also gives each region's FP64 eigen features from FP64 Hessian sums, the error reference
for the float outputs.  The shapes must satisfy the reference kernels' launch geometry
(W % 320, H % 360, D % 16 among others), which ref_cubin checks before any launch.
"""
import ctypes
import os

import numpy as np

from . import ref_cubin

HERE = os.path.dirname(os.path.abspath(__file__))
FEATURES_LIB = os.path.join(HERE, "_build", "libref_features.so")

DT_RECORD = np.dtype([
    ("local_x", "<f4"), ("local_y", "<f4"), ("local_z", "<f4"),
    ("structureness", "<f4"), ("blobness", "<f4"), ("intensity", "<f4"),
    ("size", "<u2"), ("padding", "<u2"),
])

_lib = None


def features_lib():
    global _lib
    if _lib is None:
        if not os.path.exists(FEATURES_LIB):
            from . import build_oracle
            build_oracle.build_ref_features()
        L = ctypes.CDLL(FEATURES_LIB)
        L.ref_regional_features.restype = ctypes.c_int
        L.ref_regional_features.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 4 + [ctypes.c_void_p] * 9
        _lib = L
    return _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def regional_features(labels, hessian, norm, is_ave):
    """HessianFeatures + MaxNormalized/SumNormalized + RegionalSizeAndCentroid of the
    reference, through the CUB harness -> dict of numpy arrays over the regions."""
    import torch
    D, H, W = labels.shape
    n = D * H * W
    dev = labels.device
    i32 = lambda k: torch.empty(k, dtype=torch.int32, device=dev)
    f32 = lambda k: torch.empty(k, dtype=torch.float32, device=dev)
    labels_tmp, labels_reg = i32(n), i32(n)
    values_tmp, grid = f32(n), f32(n)
    hess_reg, intensity_reg, centroid_reg = f32(6 * n), f32(n), f32(3 * n)
    size_reg = torch.empty(n, dtype=torch.int16, device=dev)
    num = torch.zeros(1, dtype=torch.int32, device=dev)
    rc = features_lib().ref_regional_features(_ptr(labels), _ptr(hessian), _ptr(norm), W, H, D, int(bool(is_ave)),
                                              _ptr(labels_tmp), _ptr(values_tmp), _ptr(labels_reg), _ptr(grid),
                                              _ptr(hess_reg), _ptr(intensity_reg), _ptr(size_reg),
                                              _ptr(centroid_reg), _ptr(num))
    if rc != 0:
        raise RuntimeError("reference region reductions failed (cudaError %d)" % rc)
    R = int(num.item())
    return {
        "num_regions": R,
        "label": labels_reg[:R].cpu().numpy(),
        "hessian": hess_reg.view(6, n)[:, :R].cpu().numpy(),
        "intensity": intensity_reg[:R].cpu().numpy(),
        "size": size_reg[:R].cpu().numpy().view(np.uint16),
        "centroid": centroid_reg.view(3, n)[:, :R].cpu().numpy(),
    }


def hessian_sums_f64(labels, hessian, num_regions, label_of_region):
    """FP64 sums of the six Hessian planes per region (the error reference)."""
    import torch
    lab = labels.reshape(-1).long()
    # region index of every voxel: labels are the regions' ascending minimum voxel indices
    keys = torch.as_tensor(label_of_region, device=labels.device).long()
    idx = torch.searchsorted(keys, lab)
    out = torch.zeros((6, num_regions), dtype=torch.float64, device=labels.device)
    for k in range(6):
        out[k].index_add_(0, idx, hessian[k].reshape(-1).double())
    return out.cpu().numpy()


def eigen_f64(h):
    """The Eberly closed form of EigenvaluesKernel (src/3D/Eigenvalues.cu:19-96) in FP64,
    vectorised, without the float rounding of its outputs: -> (structureness, blobness)."""
    xx, xy, xz, yy, yz, zz = (np.asarray(v, np.float64) for v in h)
    maxabs = np.max(np.abs(np.stack([xx, xy, xz, yy, yz, zz])), axis=0)
    nrm = xy * xy + xz * xz + yz * yz
    with np.errstate(all="ignore"):
        t = (xx + yy + zz) / 3.0
        b00, b11, b22 = xx - t, yy - t, zz - t
        den = np.sqrt((b00 * b00 + b11 * b11 + b22 * b22 + nrm * 2.0) / 6.0)
        c00 = b11 * b22 - yz * yz
        c01 = xy * b22 - yz * xz
        c02 = xy * yz - b11 * xz
        det = (b00 * c00 - xy * c01 + xz * c02) / (den * den * den)
        ang = np.arccos(np.clip(det * 0.5, -1.0, 1.0)) / 3.0
        beta2 = np.cos(ang) * 2.0
        beta0 = np.cos(ang + 2.0 * np.pi / 3.0) * 2.0
        beta1 = -(beta0 + beta2)
        e0 = np.where(nrm > 1e-30, t + den * beta0, xx)
        e1 = np.where(nrm > 1e-30, t + den * beta1, yy)
        e2 = np.where(nrm > 1e-30, t + den * beta2, zz)
        st = e0 * e0 + e1 * e1 + e2 * e2
        bl = e2 * e2 / (e0 * e1)
    zero = maxabs < 1e-30
    return np.where(zero, 0.0, st), np.where(zero, 0.0, bl)


def save_feature_vector(f, p, depth, z0, margin):
    """saveFeatureVector (src/3D/utils.h:204-250): regions 1.. that pass the margin, size and
    intensity filter, as 28-byte records; returns (records, kept region indices)."""
    cx, cy, cz = f["centroid"]
    size, inten = f["size"], f["intensity"]
    i = np.arange(1, f["num_regions"])
    cx, cy, cz, size, inten = cx[i], cy[i], cz[i], size[i], inten[i]
    keep = ~((cz < np.float32(margin)) | (cz >= np.float32(depth - margin)))
    keep &= ~((cx < np.float32(p.left_margin)) | (cx >= np.float32(p.width - p.right_margin)))
    keep &= ~((cy < np.float32(p.top_margin)) | (cy >= np.float32(p.height - p.bottom_margin)))
    keep &= ~((size < p.min_size) | (inten <= np.float32(0)))
    rows = i[keep]
    rec = np.zeros(len(rows), DT_RECORD)
    rec["local_x"] = cx[keep]
    rec["local_y"] = cy[keep]
    rec["local_z"] = (cz[keep] + np.float32(z0)).astype(np.float32)
    st, bl = f["eigen"]
    rec["structureness"] = st[rows]
    rec["blobness"] = bl[rows]
    rec["intensity"] = inten[keep]
    rec["size"] = size[keep]
    return rec, rows


def substack(img, depth_valid, z0, p, taps_fn, normalizer, margin):
    """processSubstack (HDoG3D_main.cpp:134-257) on a uint16 CUDA tensor (D, H, W) whose slices
    from depth_valid on are zero -> (records, FP64 structureness and blobness of the kept
    regions, the intermediate volumes)."""
    norm = ref_cubin.normalize(img, p.radius_norm_xy, p.radius_norm_z, float(p.min_intensity))
    dogv = ref_cubin.dog(norm, (p.sigma_xy_small, p.sigma_z_small, p.sigma_xy_large, p.sigma_z_large), taps_fn,
                         normalizer)
    hess, pd = ref_cubin.hessian_pd(dogv)
    labels, _ = ref_cubin.ccl(pd)
    f = regional_features(labels, hess, norm, p.is_ave_mode)
    f["eigen"] = ref_cubin.eigen(f["hessian"])
    rec, rows = save_feature_vector(f, p, depth_valid, z0, margin)
    h64 = hessian_sums_f64(labels, hess, f["num_regions"], f["label"])
    st64, bl64 = eigen_f64(h64[:, rows])
    return rec, (st64, bl64), {"norm": norm, "dog": dogv, "pd": pd, "labels": labels}


def stack(vol_dev, p, taps_fn, normalizer, margin, schedule):
    """The substack loop of main (HDoG3D_main.cpp:294-315) over a uint16 CUDA tensor
    (length, H, W) -> (records, FP64 structureness, FP64 blobness), substack by substack."""
    import torch
    L = vol_dev.shape[0]
    recs, st, bl = [], [], []
    for z0 in schedule:
        dv = min(p.depth, L - z0)
        sub = torch.zeros((p.depth,) + tuple(vol_dev.shape[1:]), dtype=torch.uint16, device=vol_dev.device)
        sub[:dv] = vol_dev[z0:z0 + dv]
        r, (s64, b64), _ = substack(sub, dv, z0, p, taps_fn, normalizer, margin)
        recs.append(r)
        st.append(s64)
        bl.append(b64)
    return np.concatenate(recs), np.concatenate(st), np.concatenate(bl)
