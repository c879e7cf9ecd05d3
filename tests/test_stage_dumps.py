"""The stage programs (Normalize_test, DoG_test, Hessian_test, CCL_test, Regional_test), run
as script/HDoG_intermediate.py:25-104 runs the reference's test/*_test binaries: one
parameter file holding one stack of `depth` slices, outputs written as raw volumes.

CPU: the argument and parameter-file checks that end the programs before any device work
(exit 2, as test/*_test.cpp do).  GPU: every file each program writes, bit-exact against
the oracle (structureness / blobness within the stated relative tolerance of the
float-sum oracle), and the output-name rules of the argument count and `verbose`.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from helpers import CFG_PARAMS, volume
from oracle import oracle as orc

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cubic-informatics_gb300")
TOOLS = os.path.join(PKG, "_build", "test")
EIGEN_RTOL = 1e-4      # structureness / blobness vs the float-sum oracle

W, H, D = 160, 120, 16


def write_stack(root, vol, n=None):
    """Slices {root}/stack/{z:06d}.bin (uint16, H x W) -> their paths."""
    d = os.path.join(root, "stack")
    os.makedirs(d, exist_ok=True)
    paths = []
    for z in range(vol.shape[0] if n is None else n):
        p = os.path.join(d, "%06d.bin" % z)
        np.ascontiguousarray(vol[z % vol.shape[0]]).tofile(p)
        paths.append(p)
    return paths


def write_param(path, srcs_list, verbose=0, **kw):
    """A parameter file in the reference's format (src/3D/utils.h:95-157)."""
    c = dict(CFG_PARAMS)
    c.update(kw)
    doc = {
        "devID": 0, "verbose": verbose, "is_ave_mode": c["is_ave_mode"],
        "input_image_info": {"width": W, "height": H, "left_margin": 0, "right_margin": 0,
                             "top_margin": 0, "bottom_margin": 0},
        "coordinate_info": {"scale_x": 1.0, "scale_y": 1.0, "scale_z": 1.0},
        "HDoG_param": {"depth": D, "extra_depth_margin": c["extra_depth_margin"],
                       "radius_norm": {"xy_large": c["radius_norm_xy"], "z_large": c["radius_norm_z"]},
                       "min_intensity": c["min_intensity"], "gamma_n": c["gamma_n"],
                       "sigma_dog": {"xy_small": c["sigma_xy_small"], "z_small": c["sigma_z_small"],
                                     "xy_large": c["sigma_xy_large"], "z_large": c["sigma_z_large"]},
                       "min_size": c["min_size"]},
        "stacks": [{"dst_path": os.path.join(os.path.dirname(path), "out_%d.bin" % i), "src_paths": s}
                   for i, s in enumerate(srcs_list)],
    }
    with open(path, "w") as f:
        json.dump(doc, f, indent=2)
    return path


def run(tool, args, cwd):
    exe = os.path.join(TOOLS, tool)
    assert os.path.exists(exe), "stage programs are not built (%s)" % exe
    r = subprocess.run([exe] + list(args), cwd=cwd, capture_output=True, text=True, timeout=600)
    return r.returncode, r.stdout + r.stderr


def load(path, dtype, shape):
    a = np.fromfile(path, dtype)
    assert a.size == int(np.prod(shape)), (path, a.size, shape)
    return a.reshape(shape)


def assert_bits_equal(got, ref, what):
    g, r = np.ascontiguousarray(got), np.ascontiguousarray(ref)
    if g.dtype == np.float32:
        g, r = g.view(np.uint32), r.view(np.uint32)
    bad = np.count_nonzero(g != r)
    assert bad == 0, "%s: %d of %d values differ" % (what, bad, g.size)


# ---------------------------------------------------------------- CPU: argument checks

@pytest.mark.parametrize("tool", ["Normalize_test", "DoG_test", "Hessian_test", "CCL_test", "Regional_test"])
def test_two_stacks_exit_2(tmp_path, tool):
    vol = np.zeros((D, H, W), np.uint16)
    s = write_stack(str(tmp_path), vol)
    param = write_param(str(tmp_path / "p.json"), [s, s])
    rc, out = run(tool, [param], str(tmp_path))
    assert rc == 2 and "A single stack should be provided!" in out


@pytest.mark.parametrize("tool", ["Normalize_test", "Regional_test"])
def test_wrong_depth_exit_2(tmp_path, tool):
    vol = np.zeros((D, H, W), np.uint16)
    s = write_stack(str(tmp_path), vol, n=D - 3)
    param = write_param(str(tmp_path / "p.json"), [s])
    rc, out = run(tool, [param], str(tmp_path))
    assert rc == 2 and "depth(=%d) should be %d" % (D - 3, D) in out


def test_usage_and_unreadable_param_exit_2(tmp_path):
    rc, out = run("DoG_test", [], str(tmp_path))
    assert rc == 2 and "Usage" in out
    rc, out = run("DoG_test", [str(tmp_path / "missing.json")], str(tmp_path))
    assert rc == 2 and "Unable to open file" in out
    # the generic name takes the program's name as its first argument
    rc, out = run(os.path.join("..", "hdog_stage_test"), ["CCL_test"], str(tmp_path))
    assert rc == 2 and "Usage" in out


# ---------------------------------------------------------------- GPU: the dumps

@pytest.fixture(scope="module")
def case(tmp_path_factory):
    root = tmp_path_factory.mktemp("stage")
    vol = volume(W, H, D, n_nuclei=60)
    srcs = write_stack(str(root), vol)
    c = CFG_PARAMS
    norm, ero, dil = orc.normalize(vol, c["radius_norm_xy"], c["radius_norm_z"], float(c["min_intensity"]),
                                   want_parts=True)
    dog = orc.dog(norm, c["sigma_xy_small"], c["sigma_z_small"], c["sigma_xy_large"], c["sigma_z_large"],
                  c["gamma_n"])
    mask, hess = orc.hessian_pd(dog, want_hessian=True)
    labels, n = orc.ccl(mask)
    regs = orc.regions(labels, norm, dog)
    return dict(root=root, srcs=srcs, vol=vol, norm=norm, ero=ero, dil=dil, dog=dog, mask=mask, hess=hess,
                labels=labels, n=n, regs=regs)


def workdir(case, name, verbose=0, **kw):
    d = case["root"] / name
    d.mkdir()
    return d, write_param(str(d / "param.json"), [case["srcs"]], verbose=verbose, **kw)


@pytest.mark.gpu
def test_normalize_dump_verbose(case):
    d, param = workdir(case, "norm_v", verbose=1)
    rc, out = run("Normalize_test", [param], str(d))
    assert rc == 0, out
    assert sorted(os.listdir(d)) == ["dilation_l.bin", "erosion_l.bin", "normalized.bin", "param.json"]
    assert_bits_equal(load(d / "normalized.bin", np.float32, (D, H, W)), case["norm"], "normalized")
    assert_bits_equal(load(d / "erosion_l.bin", np.float32, (D, H, W)), case["ero"], "erosion_l")
    assert_bits_equal(load(d / "dilation_l.bin", np.float32, (D, H, W)), case["dil"], "dilation_l")
    # three names: erosion, dilation, normalized in that order
    rc, out = run("Normalize_test", [param, "e.bin", "l.bin", "n.bin"], str(d))
    assert rc == 0, out
    assert_bits_equal(load(d / "e.bin", np.float32, (D, H, W)), case["ero"], "erosion (named)")
    assert_bits_equal(load(d / "l.bin", np.float32, (D, H, W)), case["dil"], "dilation (named)")
    assert_bits_equal(load(d / "n.bin", np.float32, (D, H, W)), case["norm"], "normalized (named)")


@pytest.mark.gpu
def test_normalize_dump_quiet_named(case):
    d, param = workdir(case, "norm_q")
    rc, out = run("Normalize_test", [param, "n.bin"], str(d))
    assert rc == 0, out
    assert sorted(os.listdir(d)) == ["n.bin", "param.json"]
    assert_bits_equal(load(d / "n.bin", np.float32, (D, H, W)), case["norm"], "normalized")


@pytest.mark.gpu
def test_normalize_dump_copy_path(case):
    """radius 0 skips the min/max boxes: the normalized volume is the thresholded image."""
    d, param = workdir(case, "norm_r0", radius_norm_xy=0, min_intensity=120)
    rc, out = run("Normalize_test", [param], str(d))
    assert rc == 0, out
    ref = orc.normalize(case["vol"], 0, CFG_PARAMS["radius_norm_z"], 120.0)
    assert_bits_equal(load(d / "normalized.bin", np.float32, (D, H, W)), ref, "normalized (r=0)")


@pytest.mark.gpu
def test_dog_dump(case):
    d, param = workdir(case, "dog", verbose=1)
    rc, out = run("DoG_test", [param], str(d))
    assert rc == 0, out
    assert sorted(os.listdir(d)) == ["dog.bin", "normalized.bin", "param.json"]
    assert_bits_equal(load(d / "dog.bin", np.float32, (D, H, W)), case["dog"], "dog")
    assert_bits_equal(load(d / "normalized.bin", np.float32, (D, H, W)), case["norm"], "normalized")
    rc, out = run("DoG_test", [param, "a.bin", "b.bin"], str(d))
    assert rc == 0, out
    assert_bits_equal(load(d / "a.bin", np.float32, (D, H, W)), case["norm"], "normalized (named)")
    assert_bits_equal(load(d / "b.bin", np.float32, (D, H, W)), case["dog"], "dog (named)")
    rc, out = run("DoG_test", [param, "c.bin"], str(d))
    assert rc == 0, out
    assert_bits_equal(load(d / "c.bin", np.float32, (D, H, W)), case["dog"], "dog (one name)")


@pytest.mark.gpu
def test_hessian_dump(case):
    d, param = workdir(case, "hess")
    rc, out = run("Hessian_test", [param], str(d))
    assert rc == 0, out
    assert sorted(os.listdir(d)) == ["dog.bin", "hessian_pd.bin", "param.json"]
    assert_bits_equal(load(d / "dog.bin", np.float32, (D, H, W)), case["dog"], "dog")
    assert_bits_equal(load(d / "hessian_pd.bin", np.uint8, (D, H, W)), case["mask"], "hessian_pd")


@pytest.mark.gpu
def test_hessian_dump_verbose(case):
    d, param = workdir(case, "hess_v", verbose=1)
    # verbose with fewer than two output names writes nothing (test/Hessian_test.cpp)
    rc, out = run("Hessian_test", [param], str(d))
    assert rc == 0, out
    assert sorted(os.listdir(d)) == ["param.json"]
    rc, out = run("Hessian_test", [param, "g.bin", "m.bin"], str(d))
    assert rc == 0, out
    assert_bits_equal(load(d / "g.bin", np.float32, (D, H, W)), case["dog"], "dog")
    assert_bits_equal(load(d / "m.bin", np.uint8, (D, H, W)), case["mask"], "hessian_pd")
    assert_bits_equal(load(d / "hessian.bin", np.float32, (6, D, H, W)), case["hess"], "hessian planes")
    # three names, as script/HDoG_intermediate.py passes them: dog, pd, the six planes
    rc, out = run("Hessian_test", [param, "g3.bin", "m3.bin", "h3.bin"], str(d))
    assert rc == 0, out
    assert_bits_equal(load(d / "m3.bin", np.uint8, (D, H, W)), case["mask"], "hessian_pd (3 names)")
    assert_bits_equal(load(d / "h3.bin", np.float32, (6, D, H, W)), case["hess"], "hessian planes (3 names)")


@pytest.mark.gpu
def test_ccl_dump(case):
    d, param = workdir(case, "ccl")
    rc, out = run("CCL_test", [param], str(d))
    assert rc == 0, out
    assert_bits_equal(load(d / "labels.bin", np.int32, (D, H, W)), case["labels"], "labels")
    assert_bits_equal(load(d / "hessian_pd.bin", np.uint8, (D, H, W)), case["mask"], "hessian_pd")


@pytest.mark.gpu
def test_regional_dump(case):
    d, param = workdir(case, "reg")
    rc, out = run("Regional_test", [param], str(d))
    assert rc == 0, out
    R = case["regs"]
    n = R["num_regions"]
    assert n > 20 and "num_regions: %d" % n in out
    assert_bits_equal(load(d / "labels.bin", np.int32, (D, H, W)), case["labels"], "labels")
    assert_bits_equal(load(d / "normalized.bin", np.float32, (D, H, W)), case["norm"], "normalized")
    m = n - 1
    assert_bits_equal(load(d / "labels_region.bin", np.int32, (m,)), R["label"][1:], "labels_region")
    assert_bits_equal(load(d / "size_region.bin", np.uint16, (m,)),
                      (R["count"][1:] & 0xFFFF).astype(np.uint16), "size_region")
    assert_bits_equal(load(d / "max_normalized_region.bin", np.float32, (m,)), R["max_norm"][1:],
                      "max_normalized_region")
    c16 = (R["count"][1:] & 0xFFFF).astype(np.float32)
    for k, f in enumerate(("centroid_x.bin", "centroid_y.bin", "centroid_z.bin")):
        ref = (R["sum_xyz"][k, 1:].astype(np.float32) / c16).astype(np.float32)
        assert_bits_equal(load(d / f, np.float32, (m,)), ref, f)
    st = load(d / "structureness_region.bin", np.float32, (m,)).astype(np.float64)
    bl = load(d / "blobness_region.bin", np.float32, (m,)).astype(np.float64)
    ref = np.array([orc.eigen(R["hess_f32"][:, i]) for i in range(1, n)], np.float64).reshape(m, 2)
    for got, want, name in ((st, ref[:, 0], "structureness"), (bl, ref[:, 1], "blobness")):
        fin = np.isfinite(want)
        assert np.array_equal(np.isfinite(got), fin), name
        rel = np.abs(got[fin] - want[fin]) / np.maximum(np.abs(want[fin]), 1e-30)
        assert rel.max(initial=0) <= EIGEN_RTOL, (name, float(rel.max(initial=0)))
