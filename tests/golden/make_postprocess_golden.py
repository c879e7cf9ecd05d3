"""Generates tests/golden/postprocess_golden.npz by running the reference's own record
post-processing code: HDoGResultStack (script/HalfBrainCells.py:23-56), the scale-merge
process_stack (script/MergeBrain.py:546-570) and get_X_3d (script/HDoG_classifier.py:158-176).

The modules themselves import packages this container lacks (pandas, tifffile, seaborn,
graphviz, docopt), so the generator compiles just those definitions from the reference
sources and runs them with NumPy; joblib.dump (the process_stack output) is captured.
Run in the build container, where the reference checkout exists:

    python tests/golden/make_postprocess_golden.py [REFERENCE_DIR]

NumPy here is >= 2 (float64 scalars promote float32 arrays).  NumPy 1.x value-based casting
(the "f32" mode) is reproduced by passing the float64 scalars as float32, which makes the
same expressions compute in float32.
"""
import ast
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HDOG_REFERENCE", "/root/reference")
SCRIPT = os.path.join(REF, "script")

DT_LOCAL = np.dtype([("local_x", "f4"), ("local_y", "f4"), ("local_z", "f4"), ("structureness", "f4"),
                     ("blobness", "f4"), ("intensity", "f4"), ("size", "u2"), ("padding", "u2")])
DT_GLOBAL = np.dtype([("merged_x", "f4"), ("merged_y", "f4"), ("merged_z", "f4"),
                      ("i_x", "u1"), ("i_y", "u1"), ("FWRV", "u1")])
DT_SCALEMERGED = np.dtype([("scaled_x", "f4"), ("scaled_y", "f4"), ("scaled_z", "f4"), ("is_valid", "bool")])


def ref_definition(fname, name, namespace):
    """Compiles the definition `name` (top level or nested) from a reference script."""
    path = os.path.join(SCRIPT, fname)
    tree = ast.parse(open(path).read(), path)
    for node in ast.walk(tree):
        if isinstance(node, (ast.FunctionDef, ast.ClassDef)) and node.name == name:
            exec(compile(ast.Module(body=[node], type_ignores=[]), path, "exec"), namespace)
            return namespace[name]
    raise KeyError(name)


def main():
    rng = np.random.default_rng(20261203)
    n = 600
    rec = np.zeros(n, DT_LOCAL)
    rec["local_x"] = rng.uniform(0, 2560, n).astype(np.float32)
    rec["local_y"] = rng.uniform(0, 2160, n).astype(np.float32)
    rec["local_z"] = rng.uniform(0, 1600, n).astype(np.float32)
    rec["structureness"] = np.exp(rng.normal(-6, 3, n)).astype(np.float32)
    rec["blobness"] = rng.normal(0.5, 2.0, n).astype(np.float32)
    rec["intensity"] = rng.uniform(0, 3, n).astype(np.float32)
    rec["size"] = rng.integers(0, 4000, n).astype(np.uint16)
    # edge values: zero and negative features (log10 -> -inf / NaN), zero size (division)
    rec["intensity"][:4] = [0.0, 1.0, 2.5, 0.0]
    rec["blobness"][:4] = [0.0, -1.0, np.inf, 1e-30]
    rec["structureness"][:4] = [0.0, 3.0, 1e-38, 0.0]
    rec["size"][:4] = [0, 1, 0, 7]
    rec["local_z"][4:8] = [0.0, 100.0, 100.25, 1599.5]

    # ---- HDoGResultStack
    ns = {"np": np, "os": os, "dt_local": DT_LOCAL, "dt_global": DT_GLOBAL}
    HDoGResultStack = ref_definition("HalfBrainCells.py", "HDoGResultStack", ns)
    tmp = tempfile.mkdtemp()
    rfile = os.path.join(tmp, "records.bin")
    rec.tofile(rfile)
    glob_cases = [
        dict(offset=[12345.678, -2048.3125, 7.000001], scales=[1.0, 1.0, 2.5], image_size=[2560, 2160], is_fw=True,
             i_xy=[3, 11]),
        dict(offset=[-1.1, 5000.9, 1234.5678], scales=[-0.65, -0.65, -2.5], image_size=[2560, 2160], is_fw=False,
             i_xy=[0, 127]),
    ]
    out = {"records": rec.view(np.uint8), "n": n}
    cases = {"global": [], "scalemerge": [], "clf": []}
    globals_by_mode = {}
    for gi, c in enumerate(glob_cases):
        for promote in ("f64", "f32"):
            cast = np.float64 if promote == "f64" else np.float32
            stack = types.SimpleNamespace(offset_x=cast(c["offset"][0]), offset_y=cast(c["offset"][1]),
                                          offset_z=cast(c["offset"][2]))
            r = HDoGResultStack(rfile, stack, c["is_fw"], c["i_xy"], c["scales"], c["image_size"])
            key = "global_%d_%s" % (gi, promote)
            out[key] = r.data_global.view(np.uint8)
            globals_by_mode[(gi, promote)] = r.data_global
            cases["global"].append(dict(c, promote=promote, key=key))

    # ---- process_stack (scale merge)
    dumped = {}
    joblib = types.SimpleNamespace(dump=lambda obj, path, compress=0: dumped.__setitem__(path, obj.copy()))
    ns = {"np": np, "dt_scalemerged": DT_SCALEMERGED, "joblib": joblib, "print": lambda *a, **k: None}
    process_stack = ref_definition("MergeBrain.py", "process_stack", ns)
    flip_x = np.eye(3)
    flip_x[0, :] *= -1
    swap = np.array([[0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, -1.0]])
    sm_cases = [
        dict(g=0, bound_z=[-np.inf, np.inf], margin_left=0, margin_top=0, offset=[12345.678, -2048.3125, 7.000001],
             coeff=[0.25, 0.25, 0.4], A=np.eye(3).tolist(), b=[0.0, 0.0, 0.0]),
        dict(g=0, bound_z=[3000.25, 507.0000001], margin_left=13, margin_top=-7, offset=[12000.5, -2100.0, 0.0],
             coeff=[0.1234567, 0.0987654, 1.0 / 3.0], A=flip_x.tolist(), b=[4321.0, 0.0, 0.0]),
        dict(g=1, bound_z=[257.0, np.inf], margin_left=2, margin_top=5, offset=[-1000.0, 3333.3, 1234.5678],
             coeff=[0.5, 0.5, 0.2], A=swap.tolist(), b=[0.0, 0.0, 900.0]),
    ]
    for si, c in enumerate(sm_cases):
        for promote in ("f64", "f32"):
            cast = np.float64 if promote == "f64" else np.float32
            cell = types.SimpleNamespace(data_global=globals_by_mode[(c["g"], promote)])
            bz = tuple(cast(v) if np.isfinite(v) else v for v in c["bound_z"])
            key = "scalemerge_%d_%s" % (si, promote)
            process_stack(key, cell, bz, c["margin_left"], c["margin_top"], cast(c["offset"][0]),
                          cast(c["offset"][1]), cast(c["offset"][2]), c["coeff"][0], c["coeff"][1], c["coeff"][2],
                          np.array(c["A"]), np.array(c["b"]))
            out[key] = dumped[key].view(np.uint8)
            cases["scalemerge"].append(dict(c, promote=promote, key=key,
                                            input="global_%d_%s" % (c["g"], promote)))

    # ---- get_X_3d
    ns = {"np": np}
    get_X_3d = ref_definition("HDoG_classifier.py", "get_X_3d", ns)
    clf_cases = [dict(), dict(is_ave=True),
                 dict(bias=[1.0, -2.0, 0.5], scale=[2.0, 0.5, -1.0], bias_before_log=[1e-3, 0.0, 2.0])]
    for ci, c in enumerate(clf_cases):
        kw = {k: (np.array(v) if isinstance(v, list) else v) for k, v in c.items()}
        key = "clf_%d" % ci
        out[key] = get_X_3d(rec, **kw)
        cases["clf"].append(dict(c, key=key))

    out["cases"] = np.array(json.dumps(cases))
    path = os.path.join(HERE, "postprocess_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
