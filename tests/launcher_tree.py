"""A small synthetic source tree in the launcher's layout {src_basedir}/{Y}/{Y}_{X}/{Z}.bin
(script/HDoG_gpu.py:57-66) with its run parameter file, shared by the launcher tests and
their fixture generator.  Stacks have distinct slice counts, so the launcher's sort by
count fixes their order whatever order the file system lists them in."""
import json
import os

import numpy as np

import hdog
from hdog import synth

W, H = 128, 96
GPUS = [0, 1]
# (Y, X, slices, seed)
STACKS = [["095000", "150000", 61, 11], ["095000", "160000", 47, 12], ["105000", "150000", 70, 13],
          ["105000", "160000", 38, 14], ["115000", "150000", 55, 15]]


def params():
    return hdog.make_params(width=W, height=H, depth=32, left_margin=4, right_margin=4, top_margin=4,
                            bottom_margin=4, extra_depth_margin=3, radius_norm_xy=20, radius_norm_z=5,
                            min_intensity=50, gamma_n=1.0, sigma_xy_small=2.0, sigma_z_small=1.5,
                            sigma_xy_large=3.2, sigma_z_large=2.4, min_size=0, is_ave_mode=0)


def stack_volume(length, seed):
    return synth.volume(synth.spec(W, H, length, max(1, W * H * length // 10500), synth.SEED_BASE + 500 + seed))


def build(root):
    """Writes the tree under root/src and the run's parameter file root/param.json; returns
    the parameter file's path."""
    src = os.path.join(root, "src")
    for y, x, n, seed in STACKS:
        d = os.path.join(src, y, "%s_%s" % (y, x))
        os.makedirs(d, exist_ok=True)
        vol = stack_volume(n, seed)
        for z in range(n):
            vol[z].tofile(os.path.join(d, "%06d.bin" % (200000 + 10 * z)))
    path = os.path.join(root, "param.json")
    hdog.write_param_file(path, params(), [], gpus=GPUS)
    d = json.load(open(path))
    d["src_basedir"] = src
    d["dst_basedir"] = os.path.join(root, "result")
    with open(path, "w") as f:
        json.dump(d, f, indent=2)
    return path


def relative(obj, root):
    """obj with every string path under root written as {ROOT}/..."""
    if isinstance(obj, dict):
        return {k: relative(v, root) for k, v in obj.items()}
    if isinstance(obj, list):
        return [relative(v, root) for v in obj]
    if isinstance(obj, str) and obj.startswith(root):
        return "{ROOT}" + obj[len(root):]
    return obj


def absolute(obj, root):
    if isinstance(obj, dict):
        return {k: absolute(v, root) for k, v in obj.items()}
    if isinstance(obj, list):
        return [absolute(v, root) for v in obj]
    if isinstance(obj, str) and obj.startswith("{ROOT}"):
        return root + obj[len("{ROOT}"):]
    return obj
