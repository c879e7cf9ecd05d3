"""The per-record steps after the records: local -> global coordinates (HDoGResultStack,
script/HalfBrainCells.py:44-56), the scale-merge validity and coordinates (process_stack,
script/MergeBrain.py:546-570) and the classifier features (get_X_3d,
script/HDoG_classifier.py:158-176).

Golden vectors: tests/golden/postprocess_golden.npz, written by running the reference's
own definitions (tests/golden/make_postprocess_golden.py), in both NumPy promotion modes.
CPU: the oracle restatement reproduces them bit for bit.  GPU: libhdog's kernels reproduce
the float32 / bool outputs bit for bit and the float64 features within 4 ulp (CUDA's
log10 and the host libm's are each within 1-2 ulp of the exact value); the special values
of nan_to_num (0, +-DBL_MAX) are exact.
"""
import json
import os

import numpy as np
import pytest

from oracle import postprocess as pp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "postprocess_golden.npz")


@pytest.fixture(scope="module")
def golden():
    g = np.load(GOLDEN)
    cases = json.loads(str(g["cases"]))
    rec = g["records"].view(pp.DT_LOCAL)
    assert len(rec) == int(g["n"])
    return g, cases, rec


def as_global(g, key):
    return g[key].view(pp.DT_GLOBAL)


def bits_equal(a, b):
    return a.tobytes() == b.tobytes()


def test_oracle_global_matches_reference(golden):
    g, cases, rec = golden
    for c in cases["global"]:
        got = pp.records_to_global(rec, c["offset"], c["scales"], c["image_size"], c["is_fw"], c["i_xy"], c["promote"])
        assert bits_equal(got, as_global(g, c["key"])), c["key"]


def test_oracle_scale_merge_matches_reference(golden):
    g, cases, rec = golden
    for c in cases["scalemerge"]:
        got = pp.scale_merge(as_global(g, c["input"]), c["bound_z"], c["margin_left"], c["margin_top"], c["offset"],
                             c["coeff"], c["A"], c["b"], c["promote"])
        assert bits_equal(got, g[c["key"]].view(pp.DT_SCALEMERGED)), c["key"]


def test_oracle_classifier_features_match_reference(golden):
    g, cases, rec = golden
    for c in cases["clf"]:
        kw = {k: v for k, v in c.items() if k != "key"}
        with np.errstate(all="ignore"):
            got = pp.classifier_features(rec, **kw)
        assert bits_equal(got, g[c["key"]]), c["key"]


def test_promotion_modes_differ():
    """The two NumPy generations round a float64 offset differently (the reason for the mode)."""
    rec = np.zeros(1, pp.DT_LOCAL)
    rec["local_x"] = 1.0
    off = [2.0 ** 24 + 1, 0, 0]   # not a float32: rounds to 2^24 before a float32 add
    a = pp.records_to_global(rec, off, [1.0, 1.0, 1.0], [10, 10], True, [0, 0], "f64")
    b = pp.records_to_global(rec, off, [1.0, 1.0, 1.0], [10, 10], True, [0, 0], "f32")
    assert a["merged_x"][0] == np.float32(2.0 ** 24 + 2)
    assert b["merged_x"][0] == np.float32(2.0 ** 24)


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_gpu_global_matches_reference(golden):
    import hdog
    g, cases, rec = golden
    for c in cases["global"]:
        got = hdog.records_to_global(rec.view(hdog.DT_LOCAL), c["offset"], c["scales"], c["image_size"], c["is_fw"],
                                     c["i_xy"], c["promote"])
        assert bits_equal(got, as_global(g, c["key"])), c["key"]


@pytest.mark.gpu
def test_gpu_scale_merge_matches_reference(golden):
    import hdog
    g, cases, rec = golden
    for c in cases["scalemerge"]:
        got = hdog.scale_merge(as_global(g, c["input"]).view(hdog.DT_GLOBAL), c["bound_z"], c["margin_left"],
                               c["margin_top"], c["offset"], c["coeff"], c["A"], c["b"], c["promote"])
        assert bits_equal(got, g[c["key"]].view(pp.DT_SCALEMERGED)), c["key"]


@pytest.mark.gpu
def test_gpu_classifier_features_match_reference(golden):
    """Tolerance: 4 ulp of the log10 value (the two libraries' bounds added), carried
    through `+ bias` and `* scale`, plus the rounding of those two steps."""
    import hdog
    g, cases, rec = golden
    for c in cases["clf"]:
        kw = {k: v for k, v in c.items() if k != "key"}
        got = hdog.classifier_features(rec.view(hdog.DT_LOCAL), **kw)
        want = g[c["key"]]
        special = (want == 0) | (np.abs(want) == np.finfo(np.float64).max)
        assert np.array_equal(got[special], want[special]), c["key"]
        with np.errstate(all="ignore"):
            first = rec["intensity"] / rec["size"] if c.get("is_ave") else rec["intensity"]
            F = np.array([first, rec["structureness"], rec["blobness"]]).T
            L = np.log10(F + np.asarray(c.get("bias_before_log", [0.0, 0.0, 0.0]), np.float64))
        scale = np.abs(np.asarray(c.get("scale", [1.0, 1.0, 1.0]), np.float64))
        fin = ~special & np.isfinite(L)
        with np.errstate(over="ignore"):   # spacing of +-DBL_MAX entries (excluded by `special`)
            tol = 4 * np.spacing(np.abs(L)) * scale + 2 * np.spacing(np.abs(want))
        err = np.abs(got - want)
        assert np.all(err[fin] <= tol[fin]), (c["key"], float(np.max(err[fin] - tol[fin])))
        assert np.array_equal(got[~fin & ~special], want[~fin & ~special]), c["key"]


@pytest.mark.gpu
def test_gpu_empty_inputs():
    import hdog
    empty = np.zeros(0, hdog.DT_LOCAL)
    assert len(hdog.records_to_global(empty, [0, 0, 0], [1, 1, 1], [4, 4], True, [0, 0])) == 0
    assert hdog.classifier_features(empty).shape == (0, 3)
    assert len(hdog.scale_merge(np.zeros(0, hdog.DT_GLOBAL), [0, 1], 0, 0, [0, 0, 0], [1, 1, 1], np.eye(3),
                                [0, 0, 0])) == 0
