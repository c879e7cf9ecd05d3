"""TEST INFRASTRUCTURE ONLY: numpy/ctypes front end of the CPU oracle (hdog_oracle.c).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker.  The product never imports this module.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

DT_RECORD = np.dtype([
    ("local_x", "<f4"), ("local_y", "<f4"), ("local_z", "<f4"),
    ("structureness", "<f4"), ("blobness", "<f4"), ("intensity", "<f4"),
    ("size", "<u2"), ("padding", "<u2"),
])

# Contraction form of the Sylvester test that matches the reference binary
# (pd_variant = minor form + 4 * determinant form, see orc_pd_test): both minor
# products rounded and compared, the determinant as an FMA chain whose last
# subtraction is folded into the compare.  Pinned by oracle/ref_golden.py: 0 of
# 524,288 crafted near-singular matrices differ (tests/golden/ref_stages.json).
PD_VARIANT_REFERENCE = 0 + 4 * 3


class orc_params(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int), ("depth", ctypes.c_int),
        ("radius_norm_xy", ctypes.c_int), ("radius_norm_z", ctypes.c_int),
        ("min_intensity", ctypes.c_float), ("gamma_n", ctypes.c_float),
        ("sigma_xy_small", ctypes.c_float), ("sigma_z_small", ctypes.c_float),
        ("sigma_xy_large", ctypes.c_float), ("sigma_z_large", ctypes.c_float),
        ("left_margin", ctypes.c_int), ("right_margin", ctypes.c_int),
        ("top_margin", ctypes.c_int), ("bottom_margin", ctypes.c_int),
        ("extra_depth_margin", ctypes.c_int), ("min_size", ctypes.c_int),
        ("is_ave_mode", ctypes.c_int), ("pd_variant", ctypes.c_int),
    ]


class orc_regions(ctypes.Structure):
    _fields_ = [
        ("num_regions", ctypes.c_int64),
        ("label", ctypes.c_void_p), ("count", ctypes.c_void_p), ("max_norm", ctypes.c_void_p),
        ("sum_norm_f32", ctypes.c_void_p), ("sum_norm_f64", ctypes.c_void_p),
        ("sum_x", ctypes.c_void_p), ("sum_y", ctypes.c_void_p), ("sum_z", ctypes.c_void_p),
        ("hess_f32", ctypes.c_void_p), ("hess_f64", ctypes.c_void_p),
    ]


_lib = None
_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import importlib.util
            spec = importlib.util.spec_from_file_location("_orc_build", os.path.join(HERE, "build_oracle.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_gauss_taps.restype = _I
        L.orc_gauss_taps.argtypes = [_F, _P]
        L.orc_dog_normalizer.restype = _F
        L.orc_dog_normalizer.argtypes = [_F, _F, _F]
        L.orc_minmax3d_nearest.argtypes = [_P, _P, _P, _I, _I, _I, _I, _I]
        L.orc_box3d_nearest.argtypes = [_P, _P, _I, _I, _I, _I, _I]
        L.orc_normalize.argtypes = [_P, _P, _I, _I, _I, _I, _I, _F, _P, _P]
        L.orc_gauss3d.argtypes = [_P, _P, _I, _I, _I, _P, _I, _P, _I]
        L.orc_dog.argtypes = [_P, _P, _I, _I, _I, _F, _F, _F, _F, _F]
        L.orc_hessian_pd.argtypes = [_P, _P, _P, _I, _I, _I, _I]
        L.orc_pd_test.restype = _I
        L.orc_pd_test.argtypes = [_F] * 6 + [_I]
        L.orc_pd_test_planes.argtypes = [_P, ctypes.c_int64, _I, _P]
        L.orc_ccl.restype = ctypes.c_int64
        L.orc_ccl.argtypes = [_P, _P, _I, _I, _I]
        L.orc_regions_compute.restype = _I
        L.orc_regions_compute.argtypes = [_P, _P, _P, _I, _I, _I, ctypes.POINTER(orc_regions)]
        L.orc_regions_free.argtypes = [ctypes.POINTER(orc_regions)]
        L.orc_eigen.argtypes = [_P, _P, _P]
        L.orc_erosion3d_zero.argtypes = [_P, _P, _I, _I, _I, _I, _I]
        L.orc_substack.restype = ctypes.c_int64
        L.orc_substack.argtypes = [ctypes.POINTER(orc_params), _P, _I, _I, _P, ctypes.c_int64,
                                   ctypes.POINTER(ctypes.c_int64), _P, _P]
        _lib = L
    return _lib


def _c(a, dtype):
    a = np.ascontiguousarray(a, dtype)
    return a, a.ctypes.data


def gauss_taps(sigma):
    taps = np.zeros(80, np.float32)
    r = lib().orc_gauss_taps(_F(sigma), taps.ctypes.data)
    return taps, r


def dog_normalizer(sxy1, sz1, gamma):
    return lib().orc_dog_normalizer(_F(sxy1), _F(sz1), _F(gamma))


def minmax3d(img, rxy, rz):
    img, p = _c(img, np.uint16)
    D, H, W = img.shape
    ero = np.empty_like(img)
    dil = np.empty_like(img)
    lib().orc_minmax3d_nearest(p, ero.ctypes.data, dil.ctypes.data, W, H, D, rxy, rz)
    return ero, dil


def normalize(img, rxy, rz, min_intensity, want_parts=False):
    img, p = _c(img, np.uint16)
    D, H, W = img.shape
    norm = np.empty(img.shape, np.float32)
    e = np.empty(img.shape, np.float32) if want_parts else None
    d = np.empty(img.shape, np.float32) if want_parts else None
    lib().orc_normalize(p, norm.ctypes.data, W, H, D, rxy, rz, _F(min_intensity),
                        e.ctypes.data if want_parts else None, d.ctypes.data if want_parts else None)
    return (norm, e, d) if want_parts else norm


def gauss3d(src, sigma_xy, sigma_z):
    src, p = _c(src, np.float32)
    D, H, W = src.shape
    kxy, rxy = gauss_taps(sigma_xy)
    kz, rz = gauss_taps(sigma_z)
    out = np.empty_like(src)
    lib().orc_gauss3d(p, out.ctypes.data, W, H, D, kxy.ctypes.data, rxy, kz.ctypes.data, rz)
    return out


def dog(norm, sxy1, sz1, sxy2, sz2, gamma=1.0):
    norm, p = _c(norm, np.float32)
    D, H, W = norm.shape
    out = np.empty_like(norm)
    lib().orc_dog(p, out.ctypes.data, W, H, D, _F(sxy1), _F(sz1), _F(sxy2), _F(sz2), _F(gamma))
    return out


def hessian_pd(dogv, pd_variant=PD_VARIANT_REFERENCE, want_hessian=False):
    dogv, p = _c(dogv, np.float32)
    D, H, W = dogv.shape
    mask = np.empty(dogv.shape, np.uint8)
    hess = np.empty((6,) + dogv.shape, np.float32) if want_hessian else None
    lib().orc_hessian_pd(p, mask.ctypes.data, hess.ctypes.data if want_hessian else None, W, H, D, pd_variant)
    return mask, hess


def pd_test(h6, variant=PD_VARIANT_REFERENCE):
    return lib().orc_pd_test(*[_F(float(v)) for v in h6], variant)


def pd_test_planes(planes, variant=PD_VARIANT_REFERENCE):
    """Sylvester test on six planes (6, ...) -> uint8 mask of the trailing shape."""
    planes, p = _c(planes, np.float32)
    n = planes[0].size
    out = np.empty(planes.shape[1:], np.uint8)
    lib().orc_pd_test_planes(p, n, variant, out.ctypes.data)
    return out


def ccl(mask):
    mask, p = _c(mask, np.uint8)
    D, H, W = mask.shape
    labels = np.empty(mask.shape, np.int32)
    n = lib().orc_ccl(p, labels.ctypes.data, W, H, D)
    return labels, int(n)


def regions(labels, norm, dogv):
    labels, pl = _c(labels, np.int32)
    norm, pn = _c(norm, np.float32)
    dogv, pd = _c(dogv, np.float32)
    D, H, W = labels.shape
    r = orc_regions()
    if lib().orc_regions_compute(pl, pn, pd, W, H, D, ctypes.byref(r)) != 0:
        raise MemoryError("oracle regions")
    n = int(r.num_regions)

    def take(ptr, ctype, rows=1):
        a = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctype)), shape=(rows * n,)).copy()
        return a.reshape(rows, n) if rows > 1 else a

    out = {
        "num_regions": n,
        "label": take(r.label, ctypes.c_int32),
        "count": take(r.count, ctypes.c_int64),
        "max_norm": take(r.max_norm, ctypes.c_float),
        "sum_norm_f32": take(r.sum_norm_f32, ctypes.c_float),
        "sum_norm_f64": take(r.sum_norm_f64, ctypes.c_double),
        "sum_xyz": np.stack([take(r.sum_x, ctypes.c_double), take(r.sum_y, ctypes.c_double),
                             take(r.sum_z, ctypes.c_double)]),
        "hess_f32": take(r.hess_f32, ctypes.c_float, 6),
        "hess_f64": take(r.hess_f64, ctypes.c_double, 6),
    }
    lib().orc_regions_free(ctypes.byref(r))
    return out


def eigen(hs6):
    hs = np.ascontiguousarray(hs6, np.float32)
    st = np.zeros(1, np.float32)
    bl = np.zeros(1, np.float32)
    lib().orc_eigen(hs.ctypes.data, st.ctypes.data, bl.ctypes.data)
    return float(st[0]), float(bl[0])


def erosion(img, rxy, rz):
    img, p = _c(img, np.uint16)
    D, H, W = img.shape
    out = np.empty_like(img)
    lib().orc_erosion3d_zero(p, out.ctypes.data, W, H, D, rxy, rz)
    return out


def params_from(hp, pd_variant=PD_VARIANT_REFERENCE):
    """orc_params from an hdog_params-like object (attribute access)."""
    o = orc_params()
    for name, _ in orc_params._fields_:
        if name == "pd_variant":
            o.pd_variant = pd_variant
        elif name == "min_intensity":
            o.min_intensity = float(hp.min_intensity)
        else:
            setattr(o, name, getattr(hp, name))
    return o


def substack(op, img, depth_valid, z0):
    """One substack (img: depth x H x W, zero tail applied) -> (records, num_regions, mask, labels)."""
    img, p = _c(img, np.uint16)
    cap = 1 << 20
    out = np.empty(cap, DT_RECORD)
    nreg = ctypes.c_int64()
    mask = np.empty(img.shape, np.uint8)
    labels = np.empty(img.shape, np.int32)
    n = lib().orc_substack(ctypes.byref(op), p, depth_valid, z0, out.ctypes.data, cap, ctypes.byref(nreg),
                           mask.ctypes.data, labels.ctypes.data)
    if n < 0:
        raise MemoryError("oracle substack")
    return out[: min(n, cap)].copy(), int(nreg.value), mask, labels


def depth_margin(op):
    return gauss_taps(op.sigma_z_large)[1] + op.extra_depth_margin


def schedule(length, depth, margin):
    if length - margin <= 0:
        return []
    stride = depth - 2 * margin
    assert stride > 0
    return list(range(0, length - margin, stride))


def stack(op, vol):
    """All substacks of a stack in the HDoG3D_main schedule (HDoG3D_main.cpp:294-315)."""
    L = vol.shape[0]
    m = depth_margin(op)
    recs = []
    for z0 in schedule(L, op.depth, m):
        dv = min(op.depth, L - z0)
        sub = np.zeros((op.depth,) + vol.shape[1:], np.uint16)
        sub[:dv] = vol[z0:z0 + dv]
        recs.append(substack(op, sub, dv, z0)[0])
    return np.concatenate(recs) if recs else np.zeros(0, DT_RECORD)
