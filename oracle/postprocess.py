"""TEST INFRASTRUCTURE (the oracle): NumPy restatement of the per-record steps that follow
the HDoG records in the reference's scripts.  Only tests/ uses it, as the checker of
libhdog's hdog_records_to_global, hdog_scale_merge and hdog_classifier_features.

  records_to_global    HDoGResultStack.__init__      script/HalfBrainCells.py:44-56
  scale_merge          process_stack                 script/MergeBrain.py:546-570
  classifier_features  get_X_3d                      script/HDoG_classifier.py:158-176

The reference mixes NumPy float64 scalars (stack offsets, z bounds) with float32 record
fields and lets NumPy's promotion decide the arithmetic: float32 under NumPy 1.x
value-based casting ("f32"), float64 under NumPy >= 2 ("f64").  `promote` selects which;
each step below rounds exactly where the corresponding NumPy expression does.
Pinned by tests/golden/postprocess_golden.npz, made by running the reference's own
functions (tests/golden/make_postprocess_golden.py).
"""
import numpy as np

DT_LOCAL = np.dtype([("local_x", "f4"), ("local_y", "f4"), ("local_z", "f4"), ("structureness", "f4"),
                     ("blobness", "f4"), ("intensity", "f4"), ("size", "u2"), ("padding", "u2")])
DT_GLOBAL = np.dtype([("merged_x", "f4"), ("merged_y", "f4"), ("merged_z", "f4"),
                      ("i_x", "u1"), ("i_y", "u1"), ("FWRV", "u1")])
DT_SCALEMERGED = np.dtype([("scaled_x", "f4"), ("scaled_y", "f4"), ("scaled_z", "f4"), ("is_valid", "bool")])


def _scalar(v, promote):
    """A NumPy float64 scalar as each NumPy generation combines it with float32 arrays."""
    return np.float32(v) if promote == "f32" else np.float64(v)


def records_to_global(data_local, offset, scales, image_size, is_fw, i_xy, promote="f64"):
    """HalfBrainCells.py:44-56: merged = offset + local * scale (float32 product; the sum
    per `promote`), then merged -= size * scale for a negative scale."""
    width, height = image_size
    sx, sy, sz = (float(s) for s in scales)
    out = np.zeros(data_local.shape[0], dtype=DT_GLOBAL)
    out["FWRV"] = 0 if is_fw else 1
    out["i_x"] = i_xy[0]
    out["i_y"] = i_xy[1]
    out["merged_x"] = _scalar(offset[0], promote) + data_local["local_x"] * sx
    out["merged_y"] = _scalar(offset[1], promote) + data_local["local_y"] * sy
    out["merged_z"] = _scalar(offset[2], promote) + data_local["local_z"] * sz
    if sx < 0:
        out["merged_x"] -= width * sx
    if sy < 0:
        out["merged_y"] -= height * sy
    return out


def scale_merge(data_global, bound_z, margin_left, margin_top, offset, coeff, A, b, promote="f64"):
    """MergeBrain.py:546-570: validity by the z bounds, then the scaled coordinates (float32
    inner expression, float64 affine step)."""
    lo, hi = (bound_z[1], bound_z[0]) if bound_z[0] > bound_z[1] else (bound_z[0], bound_z[1])
    lo, hi = _scalar(lo, promote), _scalar(hi, promote)
    out = np.zeros(data_global.shape[0], dtype=DT_SCALEMERGED)
    out["is_valid"] = np.bitwise_and(lo <= data_global["merged_z"], data_global["merged_z"] <= hi)
    c = np.zeros((data_global.shape[0], 3), dtype=np.float32)
    c[:, 0] = (data_global["merged_x"] - _scalar(offset[0], promote)) * float(coeff[0]) - int(margin_left)
    c[:, 1] = (data_global["merged_y"] - _scalar(offset[1], promote)) * float(coeff[1]) - int(margin_top)
    c[:, 2] = (data_global["merged_z"] - _scalar(offset[2], promote)) * float(coeff[2])
    r = np.asarray(A, np.float64).dot(c.T).T + np.asarray(b, np.float64)
    out["scaled_x"] = r[:, 0]
    out["scaled_y"] = r[:, 1]
    out["scaled_z"] = r[:, 2]
    return out


def classifier_features(data, bias=(0, 0, 0), scale=(1.0, 1.0, 1.0), bias_before_log=(0.0, 0.0, 0.0), is_ave=False):
    """HDoG_classifier.py:158-176 (get_X_3d)."""
    first = data["intensity"] / data["size"] if is_ave else data["intensity"]
    F = np.array([first, data["structureness"], data["blobness"]]).T
    return np.nan_to_num((np.log10(F + np.asarray(bias_before_log, np.float64)) + np.asarray(bias)) *
                         np.asarray(scale, np.float64))
