"""The CPU oracle replayed against digests of the reference's own kernels.

tests/golden/ref_stages.json was written by oracle/ref_golden.py on a GB300, running
the reference's src/3D kernels (compiled unmodified for sm_103a) on seeded synthetic
volumes.  Here the oracle recomputes each case from the same seed and must reproduce
every stage digest bit for bit: normalized volume, DoG, the six Hessian planes, the
negative-definite mask and the CCL labels; and the erosion operator.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from hdog import synth
from oracle import oracle as orc

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_stages.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def case_volume(c):
    return synth.volume(synth.spec(c["W"], c["H"], c["D"], c["n_nuclei"], c["seed"], **c["synth"]))


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_oracle_reproduces_reference_digests(case):
    vol = case_volume(case)
    assert sha(vol) == case["sha256_input"], "synthetic generator drifted"
    sx1, sz1, sx2, sz2 = case["sigma"]
    rxy, rz = case["radius_norm"]
    norm = orc.normalize(vol, rxy, rz, case["min_intensity"])
    assert sha(norm) == case["sha256"]["norm"]
    dog = orc.dog(norm, sx1, sz1, sx2, sz2, case["gamma"])
    assert sha(dog) == case["sha256"]["dog"]
    mask, hess = orc.hessian_pd(dog, want_hessian=True)
    assert sha(hess) == case["sha256"]["hessian"]
    assert sha(mask) == case["sha256"]["pd"]
    labels, n = orc.ccl(mask)
    assert sha(labels) == case["sha256"]["labels"]
    assert n == case["num_regions"]
    # and on the GPU host the oracle matched the reference with zero differing values
    assert all(v == 0 for v in case["oracle_mismatch"].values()), case["oracle_mismatch"]
    assert case["eigen_bit_mismatch"] == {"structureness": 0, "blobness": 0}


def test_oracle_erosion_reproduces_reference_digest():
    e = GOLDEN["erosion"]
    c = [c for c in GOLDEN["cases"] if c["name"] == e["case"]][0]
    out = orc.erosion(case_volume(c), *e["radius"])
    assert sha(out) == e["sha256"] and e["oracle_mismatch"] == 0


def test_oracle_sylvester_form_matches_reference_on_near_singular_matrices():
    """524,288 Hessians built so that the 2x2 minor or the determinant sits at float32
    resolution; the reference's PositiveDefiniteKernel output digest was recorded on the
    GPU.  Only the contraction form the oracle uses reproduces it; the others miss by
    thousands of voxels (the recorded per-form counts)."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle"))
    from oracle import ref_golden
    g = GOLDEN["pd_adversarial"]
    planes = ref_golden.adversarial_hessians(g["voxels"], g["seed"]).reshape(6, 32, 128, 128)
    assert sha(planes) == g["sha256_planes"]
    m = orc.pd_test_planes(planes, orc.PD_VARIANT_REFERENCE)
    assert sha(m) == g["sha256_pd"]
    counts = g["mismatches_by_variant"]
    assert counts[str(orc.PD_VARIANT_REFERENCE)] == 0
    assert sorted(counts.values())[1] > 0


REF_RECORDS = os.path.join(os.path.dirname(__file__), "golden", "ref_records_camera.json")
EXACT = ("local_x", "local_y", "local_z", "intensity", "size", "padding")


@pytest.mark.skipif(not os.path.exists(REF_RECORDS), reason="reference-path record digests not recorded")
def test_oracle_reproduces_the_reference_path_on_a_full_camera_substack():
    """Substack 0 of the 2560 x 2160 x 128 camera stack (depth 32): the oracle's stage
    outputs and records against digests of the reference's own path
    (tests/golden/make_ref_records_golden.py: its kernels, its CUB reductions, its record
    filter, on a GB300)."""
    from types import SimpleNamespace
    g = json.load(open(REF_RECORDS))["camera"]
    p = SimpleNamespace(**g["params"])
    vol = synth.volume(synth.camera_spec(depth=128))
    sub = np.ascontiguousarray(vol[:p.depth])
    del vol
    norm = orc.normalize(sub, p.radius_norm_xy, p.radius_norm_z, float(p.min_intensity))
    assert sha(norm) == g["substack0_stage_sha256"]["norm"]
    dog = orc.dog(norm, p.sigma_xy_small, p.sigma_z_small, p.sigma_xy_large, p.sigma_z_large, p.gamma_n)
    assert sha(dog) == g["substack0_stage_sha256"]["dog"]
    del norm, dog
    rec, _, mask, labels = orc.substack(orc.params_from(p), sub, p.depth, 0)
    assert sha(mask) == g["substack0_stage_sha256"]["pd"]
    assert sha(labels) == g["substack0_stage_sha256"]["labels"]
    assert len(rec) == g["substack0_records"]
    from numpy.lib import recfunctions as rfn
    assert sha(rfn.repack_fields(rec[list(EXACT)])) == g["substack0_exact_fields_sha256"]
