"""Writes ref_records_camera.json: the records of the reference's own code path
(oracle/ref_records.py: its stage kernels compiled unmodified, its CUB region reductions,
its record filter) on the 2560 x 2160 x 128 camera stack at substack depth 32, with
digests of substack 0's stage outputs, and this library's records compared against them.
Needs a GB300 and the reference's kernels built as cubins (oracle/build_oracle.py).

    python tests/golden/make_ref_records_golden.py OUT_DIR
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cubic-informatics_gb300"))

EXACT = ("local_x", "local_y", "local_z", "intensity", "size", "padding")
CAMERA = dict(width=2560, height=2160, depth=32, left_margin=100, right_margin=100, top_margin=100,
              bottom_margin=100, extra_depth_margin=3, radius_norm_xy=20, radius_norm_z=5, min_intensity=50,
              gamma_n=1.0, sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2, sigma_z_large=2.4,
              min_size=0, is_ave_mode=0)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def exact_fields(rec):
    """The exact fields alone, packed (a multi-field view keeps the other fields' bytes)."""
    from numpy.lib import recfunctions as rfn
    return np.ascontiguousarray(rfn.repack_fields(rec[list(EXACT)]))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-30)
    return float(d.max()) if len(d) else 0.0


def compare(ours, ref, st64, bl64):
    """Record-by-record comparison: exact fields bit for bit, eigen features relative."""
    out = {"records_ours": int(len(ours)), "records_reference": int(len(ref))}
    if len(ours) != len(ref):
        out["exact_fields_equal"] = False
        return out
    out["exact_fields_equal"] = bool(exact_fields(ours).tobytes() == exact_fields(ref).tobytes())
    def bits(a):
        return a.view(np.uint32) if a.dtype.itemsize == 4 else a.view(np.uint16)
    diff = {f: bits(ours[f]) != bits(ref[f]) for f in EXACT}
    out["exact_field_mismatches"] = {f: int(d.sum()) for f, d in diff.items()}
    bad = np.zeros(len(ours), bool)
    for d in diff.values():
        bad |= d
    if bad.any():
        idx = np.nonzero(bad)[0]
        out["mismatch_region_sizes"] = sorted(int(x) for x in ref["size"][idx])[-20:]
        out["mismatch_examples"] = [dict([(f, float(ours[f][i])) for f in EXACT] +
                                         [("reference_" + f, float(ref[f][i])) for f in EXACT]) for i in idx[:5]]
    for f, f64 in (("structureness", st64), ("blobness", bl64)):
        out[f + "_max_rel_vs_reference"] = rel(ours[f], ref[f])
        out[f + "_max_rel_ours_vs_fp64"] = rel(ours[f], f64)
        out[f + "_max_rel_reference_vs_fp64"] = rel(ref[f], f64)
    return out


def camera_case():
    import torch
    import hdog
    from hdog import synth
    from oracle import ref_records
    from oracle import oracle as orc
    p = hdog.make_params(**CAMERA)
    vol = synth.volume(synth.camera_spec(depth=128))
    dev = torch.from_numpy(vol).cuda()
    op = orc.params_from(p)
    margin = orc.depth_margin(op)
    sched = orc.schedule(vol.shape[0], p.depth, margin)
    taps_fn = orc.gauss_taps
    normalizer = orc.dog_normalizer(p.sigma_xy_small, p.sigma_z_small, p.gamma_n)
    # substack 0 stage digests
    sub0 = dev[:p.depth].contiguous()
    rec0, _, vols = ref_records.substack(sub0, p.depth, 0, p, taps_fn, normalizer, margin)
    stages = {k: sha(v.cpu().numpy()) for k, v in vols.items()}
    ref, st64, bl64 = ref_records.stack(dev, p, taps_fn, normalizer, margin, sched)
    with hdog.Context(p, max_substacks=len(sched)) as ctx:
        ours = ctx.run_stack(dev)
    return {
        "workload": "camera stack uint16 2560x2160x128 (hdog.synth.camera_spec), HDoG depth 32, 8 substacks",
        "params": CAMERA,
        "substack0_stage_sha256": stages,
        "substack0_records": int(len(rec0)),
        "substack0_exact_fields_sha256": sha(exact_fields(rec0)),
        "stack_records": int(len(ref)),
        "stack_exact_fields_sha256": sha(exact_fields(ref)),
        "comparison": compare(ours, ref, st64, bl64),
    }


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    res = {"generator": "tests/golden/make_ref_records_golden.py", "camera": camera_case()}
    path = os.path.join(out_dir, "ref_records_camera.json")
    with open(path, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res["camera"]["comparison"]))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_records_golden.py OUT_DIR")
    main(sys.argv[1])
