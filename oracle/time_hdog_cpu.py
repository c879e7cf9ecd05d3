"""Times the reference's own CPU script, script/HDoG_cpu.py, as a labelled second baseline.

Test and measurement infrastructure only: it needs the reference checkout (path from the
first argument or HDOG_REFERENCE) and runs where that checkout is, not on the GPU hosts.

HDoG_cpu.py imports pandas and scikit-image, which this image lacks, so two stand-ins are
put in sys.modules before the script is loaded (its own code runs unchanged):
  pandas.DataFrame / pandas.Series -> a dict of numpy arrays / the array itself
  skimage.morphology.label         -> scipy.ndimage.label with a 3x3x3 structure
                                      (full connectivity, as skimage's default for 3-D)
scikit-learn is only used by its classifier, which is not timed.

HDoG_cpu.py is a teaching restatement with its own semantics (normalization by
I/(dil-ero) with constant-zero box borders, scipy Gaussians truncated at 2 sigma, np.gradient
Hessians, no substack margins, no record filter), so its output is not compared with the
CUDA path; only its time is reported.  numpy/scipy run it on one core.

    python oracle/time_hdog_cpu.py [REFERENCE_DIR] [--out result.json]
"""
import argparse
import importlib.util
import json
import os
import platform
import sys
import time
import types

import numpy as np
import scipy.ndimage

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cubic-informatics_gb300"))


def _install_shims():
    pd = types.ModuleType("pandas")
    pd.Series = lambda a: np.asarray(a)
    pd.DataFrame = lambda d: {k: np.asarray(v) for k, v in d.items()}
    sk = types.ModuleType("skimage")
    morph = types.ModuleType("skimage.morphology")
    morph.label = lambda img: scipy.ndimage.label(img, structure=np.ones((3, 3, 3), bool))[0]
    sk.morphology = morph
    sys.modules.setdefault("pandas", pd)
    sys.modules.setdefault("skimage", sk)
    sys.modules.setdefault("skimage.morphology", morph)


def load_reference(ref_dir):
    _install_shims()
    path = os.path.join(ref_dir, "script", "HDoG_cpu.py")
    spec = importlib.util.spec_from_file_location("hdog_cpu_reference", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def time_chain(mod, vol):
    """One pass of HDoG_cpu.py's stages over `vol` (z, y, x), with the benchmark's
    parameters: sigma xy (2.0, 3.2), z (1.5, 2.4), normalization radius xy 20 / z 5,
    min_intensity 50."""
    D, H, W = vol.shape
    h = mod.HDoG_CPU(width=W, height=H, depth=D, sigma_xy=(2.0, 3.2), sigma_z=(1.5, 2.4),
                     radius_small=(4, 2), radius_large=(20, 5), min_intensity=50, gamma=1.0)
    t = {}
    t0 = time.perf_counter()
    norm = h.Normalize(vol)
    t["Normalize"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    dog = h.DoGFilter(norm)
    t["DoGFilter"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    pd_img, hess = h.HessianPDFilter(dog)
    t["HessianPDFilter"] = time.perf_counter() - t0
    del dog
    t0 = time.perf_counter()
    labels = h.CCL(pd_img)
    t["CCL"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    df = h.RegionalFeatures(norm, hess, labels)
    t["RegionalFeatures"] = time.perf_counter() - t0
    total = sum(t.values())
    return {"shape_zyx": [D, H, W], "voxels": int(vol.size), "stage_s": {k: round(v, 3) for k, v in t.items()},
            "total_s": round(total, 3), "gvox_per_s": vol.size / total / 1e9, "regions": int(len(df["index"]))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference", nargs="?", default=os.environ.get("HDOG_REFERENCE"))
    ap.add_argument("--out")
    ap.add_argument("--skip-substack", action="store_true")
    a = ap.parse_args()
    if not a.reference:
        sys.exit("give the reference checkout as an argument or in HDOG_REFERENCE")
    from hdog import synth
    mod = load_reference(a.reference)
    res = {"script": "script/HDoG_cpu.py (unchanged; pandas and skimage.morphology.label replaced by stand-ins)",
           "host": {"machine": platform.machine(), "cpu_count": os.cpu_count(), "cores_used": 1,
                    "numpy": np.__version__, "scipy": scipy.__version__}, "runs": []}
    cube = synth.volume(synth.cube_spec())
    res["runs"].append(dict(case="cube 64x256x256 (400 nuclei)", **time_chain(mod, cube)))
    if not a.skip_substack:
        sub = synth.volume(synth.camera_spec(), 0, 32)
        res["runs"].append(dict(case="camera stack substack 0, 32x2160x2560", **time_chain(mod, sub)))
    print(json.dumps(res, indent=1))
    if a.out:
        with open(a.out, "w") as fh:
            json.dump(res, fh, indent=1)


if __name__ == "__main__":
    main()
