"""C-ABI surface of libhdog.so and the host-side logic that runs without a GPU."""
import ctypes
import json
import os
import re
import subprocess

import numpy as np
import pytest

import hdog
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "hdog.h")).read()
    return sorted(set(re.findall(r"\b(hdog_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(hdog.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python mirror binds each of them
    assert set(names) <= set(hdog._SIGNATURES), set(names) - set(hdog._SIGNATURES)


def test_struct_layouts():
    assert hdog.DT_LOCAL.itemsize == 28          # FeatureVector, src/3D/utils.h:188-197
    assert ctypes.sizeof(hdog.hdog_params) == 21 * 4
    assert hdog.lib().hdog_abi_version() == 5
    assert ctypes.sizeof(hdog.hdog_soft_params) == 5 * 4 + 4 + 6 * 4 + 2 * 4 + 3 * 4
    # the record post-processing types: packed NumPy records, plain parameter blocks
    assert hdog.DT_GLOBAL.itemsize == 15 and hdog.DT_SCALEMERGED.itemsize == 13
    assert ctypes.sizeof(hdog.hdog_global_params) == 6 * 8 + 6 * 4
    assert ctypes.sizeof(hdog.hdog_scalemerge_params) == 22 * 8 + 8
    assert ctypes.sizeof(hdog.hdog_clf_params) == 9 * 8 + 8


@pytest.mark.parametrize("sigma", [0.0, 0.4, 1.5, 1.8, 2.0, 2.4, 2.7, 3.2, 4.0, 6.0, 12.3])
def test_gaussian_taps_match_oracle(sigma):
    t, r = hdog.gaussian_taps(sigma)
    to, ro = orc.gauss_taps(sigma)
    assert r == ro == int(2.0 * sigma + 0.5)
    assert np.array_equal(t.view(np.uint32), to.view(np.uint32))
    assert abs(float(t[: 2 * r + 1].astype(np.float64).sum()) - 1.0) < 1e-6
    assert np.all(t[2 * r + 1:] == 0)


def test_gaussian_taps_reject_wide_sigma():
    with pytest.raises(hdog.HDoGError) as e:
        hdog.gaussian_taps(25.0)
    assert e.value.code == hdog.HDOG_ERR_SHAPE


def test_depth_margin():
    p = hdog.make_params(sigma_z_large=2.7, extra_depth_margin=3)
    assert hdog.depth_margin(p) == 5 + 3
    p = hdog.make_params(sigma_z_large=2.4, extra_depth_margin=3)
    assert hdog.depth_margin(p) == 5 + 3


@pytest.mark.parametrize("length,depth,margin,expect", [
    (64, 64, 8, [0, 48]),
    (128, 32, 8, [0, 16, 32, 48, 64, 80, 96, 112]),
    (8, 32, 8, []),
    (9, 32, 8, [0]),
    (100, 64, 8, [0, 48]),
])
def test_substack_schedule(length, depth, margin, expect):
    # HDoG3D_main.cpp:309-314: z0 = 0, D-2m, ... while z0 < length - m
    assert hdog.substack_schedule(length, depth, margin) == expect
    assert orc.schedule(length, depth, margin) == expect


def example_param_dict(tmp_path, stacks):
    # same keys and comment style as the reference's param/param_example_HDoG_FW.json
    return {
        "src_basedir": str(tmp_path), "dst_basedir": str(tmp_path), "gpus": [0],
        "input_image_info": {"width": 2560, "height": 2160, "#": "margin in pixels",
                             "left_margin": 100, "right_margin": 90, "top_margin": 80, "bottom_margin": 70},
        "coordinate_info": {"scale_x": -0.65, "scale_y": -0.65, "scale_z": 5.0,
                            "affine_global": [[0, 0.1, 0, 0], [0.1, 0, 0, 0], [0, 0, 5, -1e6]]},
        "HDoG_param": {"depth": 32, "extra_depth_margin": 3, "cub_tmp_size_factor": 8.001,
                       "min_intensity_skip": 1000, "radius_norm": {"xy_large": 100, "z_large": 5},
                       "min_intensity": 1000, "gamma_n": 1.0,
                       "sigma_dog": {"xy_small": 4.0, "z_small": 1.8, "xy_large": 6.0, "z_large": 2.7},
                       "min_size": 10},
        "is_ave_mode": True,
        "devID": 0,
        "stacks": stacks,
    }


def test_param_file_roundtrip(tmp_path):
    d = example_param_dict(tmp_path, [])
    f = tmp_path / "p.json"
    f.write_text(json.dumps(d))
    p = hdog.load_param_file(str(f))
    assert (p.width, p.height, p.depth) == (2560, 2160, 32)
    assert (p.left_margin, p.right_margin, p.top_margin, p.bottom_margin) == (100, 90, 80, 70)
    assert (p.radius_norm_xy, p.radius_norm_z, p.min_intensity, p.min_size) == (100, 5, 1000, 10)
    assert (p.sigma_xy_small, p.sigma_z_small, p.sigma_xy_large) == (4.0, np.float32(1.8), 6.0)
    assert p.is_ave_mode == 1 and p.extra_depth_margin == 3 and p.gamma_n == 1.0
    # the writer produces a file the reader (and the reference's loader) accepts
    g = tmp_path / "q.json"
    hdog.write_param_file(str(g), p, [("out.bin", ["a.bin", "b.bin"])])
    q = hdog.load_param_file(str(g))
    assert q.as_dict() == p.as_dict()


def test_param_file_errors(tmp_path):
    with pytest.raises(hdog.HDoGError) as e:
        hdog.load_param_file(str(tmp_path / "missing.json"))
    assert e.value.code == hdog.HDOG_ERR_IO
    d = example_param_dict(tmp_path, [])
    del d["HDoG_param"]["sigma_dog"]["z_large"]
    f = tmp_path / "p.json"
    f.write_text(json.dumps(d))
    with pytest.raises(hdog.HDoGError) as e:
        hdog.load_param_file(str(f))
    assert e.value.code == hdog.HDOG_ERR_PARAM and "z_large" in str(e.value)
    f.write_text("{ not json")
    with pytest.raises(hdog.HDoGError) as e:
        hdog.load_param_file(str(f))
    assert e.value.code == hdog.HDOG_ERR_PARAM


def test_run_param_file_reports_io_errors_without_exiting(tmp_path):
    # a missing slice is an error status, not a process exit (utils.h:163-166 exits)
    d = example_param_dict(tmp_path, [{"dst_path": str(tmp_path / "r.bin"),
                                       "src_paths": [str(tmp_path / ("nope_%03d.bin" % i)) for i in range(40)]}])
    d["input_image_info"].update(width=64, height=64, left_margin=0, right_margin=0, top_margin=0, bottom_margin=0)
    d["HDoG_param"]["radius_norm"]["xy_large"] = 10
    f = tmp_path / "p.json"
    f.write_text(json.dumps(d))
    with pytest.raises(hdog.HDoGError) as e:
        hdog.run_param_file(str(f))
    assert e.value.code in (hdog.HDOG_ERR_IO, hdog.HDOG_ERR_CUDA)


def test_hdog_main_usage_and_missing_file(tmp_path):
    r = subprocess.run([hdog.MAIN_PATH], stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 2 and b"PARAM_FILE" in r.stdout
    r = subprocess.run([hdog.MAIN_PATH, str(tmp_path / "none.json")], stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 2


def test_context_rejects_bad_geometry():
    for kw in (dict(width=1), dict(depth=0), dict(radius_norm_xy=500), dict(sigma_xy_large=30.0),
               dict(width=4096, height=4096, depth=256)):
        p = hdog.make_params(**kw)
        size = ctypes.c_size_t()
        rc = hdog.lib().hdog_ctx_bytes(ctypes.byref(p), 1, ctypes.byref(size))
        assert rc in (hdog.HDOG_ERR_SHAPE, hdog.HDOG_ERR_ARG), kw


def test_context_bytes_scale_with_substacks():
    p = hdog.make_params(width=2560, height=2160, depth=32)
    a, b = ctypes.c_size_t(), ctypes.c_size_t()
    hdog.check(hdog.lib().hdog_ctx_bytes(ctypes.byref(p), 1, ctypes.byref(a)))
    hdog.check(hdog.lib().hdog_ctx_bytes(ctypes.byref(p), 4, ctypes.byref(b)))
    n = 2560 * 2160 * 32
    assert 30 * n < a.value < 70 * n
    assert 3.9 * a.value < b.value < 4.1 * a.value


def soft_params(**kw):
    v = dict(width=44, height=40, depth=14, radius_norm_xy=4, radius_norm_z=2, min_intensity=50.0,
             sigma=[1.2, 1.3, 1.1, 1.9, 2.1, 1.7], gamma=1.0, tau=1e-3, thresh=[0.0, 0.0, 0.0])
    v.update(kw)
    return hdog.hdog_soft_params(v["width"], v["height"], v["depth"], v["radius_norm_xy"], v["radius_norm_z"],
                                 v["min_intensity"], (ctypes.c_float * 6)(*v["sigma"]), v["gamma"], v["tau"],
                                 (ctypes.c_float * 3)(*v["thresh"]))


@pytest.mark.parametrize("what,kw,ptrs,code", [
    ("no volume", {}, dict(vol=None), hdog.HDOG_ERR_ARG),
    ("no workspace", {}, dict(work=None), hdog.HDOG_ERR_ARG),
    ("negative point count", {}, dict(n_pos=-1), hdog.HDOG_ERR_ARG),
    ("points without a pointer", {}, dict(pos=None), hdog.HDOG_ERR_ARG),
    ("empty frame", dict(width=0), {}, hdog.HDOG_ERR_PARAM),
    ("tau not positive", dict(tau=0.0), {}, hdog.HDOG_ERR_PARAM),
    ("negative normalization radius", dict(radius_norm_z=-1), {}, hdog.HDOG_ERR_PARAM),
    ("sigma with taps past radius 31", dict(sigma=[1.2, 1.3, 1.1, 1.9, 2.1, 15.8]), {}, hdog.HDOG_ERR_SHAPE),
    ("sigma not positive", dict(sigma=[1.2, 0.0, 1.1, 1.9, 2.1, 1.7]), {}, hdog.HDOG_ERR_SHAPE),
])
def test_soft_entry_points_check_their_arguments_on_the_host(what, kw, ptrs, code):
    """The differentiable chain's three entry points refuse bad arguments before any device
    work (the pointers below are never dereferenced: every case fails its checks first)."""
    L = hdog.lib()
    p = soft_params(**kw)
    fake = ctypes.c_void_p(4096)
    a = dict(vol=fake, pos=fake, n_pos=3, neg=fake, n_neg=2, work=fake)
    a.update(ptrs)
    out = ctypes.c_void_p(8192)
    rc = L.hdog_soft_forward(ctypes.byref(p), a["vol"], a["pos"], a["n_pos"], a["neg"], a["n_neg"], out, None,
                             a["work"], None)
    assert rc == code, (what, rc)
    assert b"hdog_soft_forward" in L.hdog_last_error()
    for name in ("hdog_soft_backward", "hdog_soft_backward_kept"):
        rc = getattr(L, name)(ctypes.byref(p), a["vol"], a["pos"], a["n_pos"], a["neg"], a["n_neg"], 1.0, None, None,
                              None, a["work"], None)
        assert rc == code, (what, name, rc)
        assert name.encode() in L.hdog_last_error()


def test_soft_forward_needs_a_loss_pointer():
    L = hdog.lib()
    p = soft_params()
    fake = ctypes.c_void_p(4096)
    assert L.hdog_soft_forward(ctypes.byref(p), fake, fake, 1, fake, 1, None, None, fake, None) == hdog.HDOG_ERR_ARG


def test_graph_entry_points_check_their_arguments_on_the_host():
    """The batched graph form's entry points refuse missing arguments before any device work;
    destroying a null graph is a no-op."""
    L = hdog.lib()
    out = ctypes.c_void_p()
    assert L.hdog_graph_create(None, 1, None, 0, None, None) == hdog.HDOG_ERR_ARG
    assert L.hdog_graph_create(None, 1, None, 0, None, ctypes.byref(out)) == hdog.HDOG_ERR_ARG
    assert out.value is None
    ctx = (ctypes.c_void_p * 1)()
    assert L.hdog_graph_create(ctx, 0, None, 0, None, ctypes.byref(out)) == hdog.HDOG_ERR_ARG
    assert L.hdog_graph_create(ctx, 1, None, 2, None, ctypes.byref(out)) == hdog.HDOG_ERR_ARG
    assert L.hdog_graph_create(ctx, 1, None, 0, None, ctypes.byref(out)) == hdog.HDOG_ERR_ARG   # null context
    assert b"hdog_graph_create" in L.hdog_last_error()
    n = ctypes.c_int64()
    assert L.hdog_graph_run(None, None, 0, ctypes.byref(n), None, None) == hdog.HDOG_ERR_ARG
    assert L.hdog_graph_last_records(None, None, 0, ctypes.byref(n)) == hdog.HDOG_ERR_ARG
    assert L.hdog_graph_destroy(None) == hdog.HDOG_OK
