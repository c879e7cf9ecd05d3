"""The per-record steps after the HDoG records, on the GPU through libhdog's C ABI:
global coordinates (HDoGResultStack, script/HalfBrainCells.py:44-56), the scale-merge
validity and coordinates (process_stack, script/MergeBrain.py:546-570) and the classifier
features (get_X_3d, script/HDoG_classifier.py:158-176).

Each function takes and returns NumPy arrays with the reference's dtypes (dt_local,
dt_global, dt_scalemerged, float64 features).  `promote` selects how the float64 scalars
meet the float32 fields: "f64" as NumPy >= 2 computes the reference's expressions, "f32"
as NumPy 1.x value-based casting does.
"""
import ctypes

import numpy as np

from . import (DT_GLOBAL, DT_LOCAL, DT_SCALEMERGED, HDOG_PROMOTE_F32, HDOG_PROMOTE_F64, check, hdog_clf_params,
               hdog_global_params, hdog_scalemerge_params, lib)

_PROMOTE = {"f32": HDOG_PROMOTE_F32, "f64": HDOG_PROMOTE_F64}


class _Device:
    """A device copy of a host array (and an output buffer), freed on exit."""

    def __init__(self):
        self.ptrs = []

    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        check(lib().hdog_device_alloc(ctypes.byref(p), max(int(nbytes), 1)))
        self.ptrs.append(p)
        return p

    def upload(self, a):
        a = np.ascontiguousarray(a)
        p = self.alloc(a.nbytes)
        if a.nbytes:
            check(lib().hdog_memcpy(p, ctypes.c_void_p(a.ctypes.data), a.nbytes, None))
        return p

    def download(self, p, out):
        if out.nbytes:
            check(lib().hdog_memcpy(ctypes.c_void_p(out.ctypes.data), p, out.nbytes, None))
        check(lib().hdog_stream_sync(None))
        return out

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        for p in self.ptrs:
            lib().hdog_device_free(p)


def records_to_global(records, offset, scales, image_size, is_fw, i_xy, promote="f64"):
    """dt_local records -> dt_global (HDoGResultStack)."""
    assert records.dtype == DT_LOCAL
    n = len(records)
    prm = hdog_global_params(float(offset[0]), float(offset[1]), float(offset[2]), float(scales[0]),
                             float(scales[1]), float(scales[2]),
                             int(image_size[0]), int(image_size[1]), 1 if is_fw else 0, int(i_xy[0]), int(i_xy[1]),
                             _PROMOTE[promote])
    out = np.empty(n, DT_GLOBAL)
    with _Device() as d:
        src, dst = d.upload(records), d.alloc(out.nbytes)
        check(lib().hdog_records_to_global(src, n, ctypes.byref(prm), dst, None))
        return d.download(dst, out)


def scale_merge(data_global, bound_z, margin_left, margin_top, offset, coeff, A, b, promote="f64"):
    """dt_global -> dt_scalemerged (the scale merge's process_stack)."""
    assert data_global.dtype == DT_GLOBAL
    n = len(data_global)
    prm = hdog_scalemerge_params()
    prm.bound_z0, prm.bound_z1 = float(bound_z[0]), float(bound_z[1])
    prm.offset_x, prm.offset_y, prm.offset_z = (float(v) for v in offset)
    prm.coeff_x, prm.coeff_y, prm.coeff_z = (float(v) for v in coeff)
    prm.margin_left, prm.margin_top = float(margin_left), float(margin_top)
    prm.A[:] = [float(v) for v in np.asarray(A, np.float64).ravel()]
    prm.b[:] = [float(v) for v in np.asarray(b, np.float64).ravel()]
    prm.promote = _PROMOTE[promote]
    out = np.empty(n, DT_SCALEMERGED)
    with _Device() as d:
        src, dst = d.upload(data_global), d.alloc(out.nbytes)
        check(lib().hdog_scale_merge(src, n, ctypes.byref(prm), dst, None))
        return d.download(dst, out)


def classifier_features(records, bias=(0, 0, 0), scale=(1.0, 1.0, 1.0), bias_before_log=(0.0, 0.0, 0.0),
                        is_ave=False):
    """dt_local records -> X (n x 3 float64), as get_X_3d."""
    assert records.dtype == DT_LOCAL
    n = len(records)
    prm = hdog_clf_params()
    prm.bias[:] = [float(v) for v in bias]
    prm.scale[:] = [float(v) for v in scale]
    prm.bias_before_log[:] = [float(v) for v in bias_before_log]
    prm.is_ave = 1 if is_ave else 0
    out = np.empty((n, 3), np.float64)
    with _Device() as d:
        src, dst = d.upload(records), d.alloc(out.nbytes)
        check(lib().hdog_classifier_features(src, n, ctypes.byref(prm), dst, None))
        return d.download(dst, out)
