"""TEST INFRASTRUCTURE: pins the CPU oracle to the reference's own CUDA kernels and
writes the golden fixtures under tests/golden/.

Run on a GPU host with oracle/_ref/*.cubin present (built by oracle/build_oracle.py in
a checkout that has the reference sources):

    python oracle/ref_golden.py OUT_DIR

For each seeded synthetic case (shapes the reference's launch geometry accepts:
W % 640, H % 720, D % 16) it runs the reference chain -- Normalize3DFilter, DoG3DFilter,
HessianPositiveDefiniteWithElement, CCL -- and the oracle on the same input, compares
every stage bit for bit, tries each floating-point contraction form of the Sylvester
test against the reference's PositiveDefiniteKernel, checks the reference
EigenvaluesKernel against the oracle's, and records SHA-256 digests of the reference
outputs.  tests/test_cpu_golden.py replays the oracle against those digests.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cubic-informatics_gb300"))

from oracle import oracle as orc  # noqa: E402
from oracle import ref_cubin  # noqa: E402
from hdog import synth  # noqa: E402

SEED = synth.SEED_BASE
BASE = dict(sigma=(2.0, 1.5, 3.2, 2.4), rxy=20, rz=5, min_intensity=50.0, gamma=1.0)
CASES = [
    dict(name="frame640x720x16", W=640, H=720, D=16, n=700, seed=SEED + 10, synth={}, **BASE),
    dict(name="frame640x720x32_pairs_atten", W=640, H=720, D=32, n=1400, seed=SEED + 11,
         synth=dict(pair_fraction=0.1, atten_z_end=0.6, stripe_amplitude=0.05), **BASE),
    dict(name="copy_path_r0", W=640, H=720, D=16, n=700, seed=SEED + 12, synth={},
         sigma=(2.0, 1.5, 3.2, 2.4), rxy=0, rz=5, min_intensity=120.0, gamma=1.0),
    dict(name="example_radii_1280x720x16", W=1280, H=720, D=16, n=1400, seed=SEED + 13, synth={},
         sigma=(4.0, 1.8, 6.0, 2.7), rxy=100, rz=5, min_intensity=50.0, gamma=1.0),
]
PD_VARIANTS = [v + 4 * d for v in range(3) for d in range(5)]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def case_volume(c):
    s = synth.spec(c["W"], c["H"], c["D"], c["n"], c["seed"], **c["synth"])
    return synth.volume(s)


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.dtype == np.float32:
        return int(np.count_nonzero(a.view(np.uint32) != b.view(np.uint32)))
    return int(np.count_nonzero(a != b))


def adversarial_hessians(n, seed):
    """Six Hessian planes whose 2x2 minor or determinant sits at float32 resolution."""
    rng = np.random.default_rng(seed)
    out = np.empty((6, n), np.float32)
    q, _ = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    lam = -np.exp(rng.uniform(-3, 3, (n, 3)))
    kind = rng.integers(0, 3, n)
    lam[kind == 1, 2] *= rng.uniform(-1, 1, (kind == 1).sum()) * 1e-6   # det ~ 0
    A = np.einsum("nij,nj,nkj->nik", q, lam, q)
    sel = kind == 2                                                      # 2x2 minor ~ 0
    a = -np.exp(rng.uniform(-2, 2, sel.sum()))
    b = -np.exp(rng.uniform(-2, 2, sel.sum()))
    A[sel, 0, 0] = a
    A[sel, 1, 1] = b
    A[sel, 0, 1] = A[sel, 1, 0] = np.sqrt(a * b) * (1 + rng.uniform(-6e-8, 6e-8, sel.sum()))
    A[sel, 0, 2] = A[sel, 2, 0] = A[sel, 1, 2] = A[sel, 2, 1] = 0.0     # det = zz * minor
    A[sel, 2, 2] = -1.0
    for k, (i, j) in enumerate([(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]):
        out[k] = A[:, i, j]
    return out


def main(out_dir):
    import torch
    os.makedirs(out_dir, exist_ok=True)
    dev = torch.device("cuda:0")
    result = {"generator": "oracle/ref_golden.py", "gpu": torch.cuda.get_device_name(0),
              "cases": [], "pd_adversarial": {}, "eigen": {}}
    # -- contraction form of the Sylvester test, on crafted near-singular Hessians
    D, H, W = 32, 128, 128
    planes = adversarial_hessians(D * H * W, SEED + 99).reshape(6, D, H, W)
    pd_ref = ref_pd_only(torch.as_tensor(planes).to(dev)).cpu().numpy()
    counts = {}
    for v in PD_VARIANTS:
        m = orc.pd_test_planes(planes, v)
        counts[str(v)] = int(np.count_nonzero(m != pd_ref))
    result["pd_adversarial"] = {"voxels": int(D * H * W), "positives": int(pd_ref.sum()),
                                "mismatches_by_variant": counts, "sha256_pd": sha(pd_ref),
                                "sha256_planes": sha(planes), "seed": SEED + 99}
    np.savez_compressed(os.path.join(out_dir, "pd_adversarial.npz"), planes=planes, pd=pd_ref)
    print("PD variants (mismatches):", counts, flush=True)

    for c in CASES:
        t0 = time.time()
        vol = case_volume(c)
        vt = torch.as_tensor(vol).to(dev)
        sx1, sz1, sx2, sz2 = c["sigma"]
        normalizer = orc.dog_normalizer(sx1, sz1, c["gamma"])
        norm_r = ref_cubin.normalize(vt, c["rxy"], c["rz"], c["min_intensity"])
        dog_r = ref_cubin.dog(norm_r, c["sigma"], orc.gauss_taps, normalizer)
        hess_r, pd_r = ref_cubin.hessian_pd(dog_r)
        labels_r, iters = ref_cubin.ccl(pd_r)
        norm_r, dog_r, hess_r, pd_r, labels_r = (t.cpu().numpy() for t in (norm_r, dog_r, hess_r, pd_r, labels_r))
        norm_o = orc.normalize(vol, c["rxy"], c["rz"], c["min_intensity"])
        dog_o = orc.dog(norm_r, sx1, sz1, sx2, sz2, c["gamma"])
        mask_o, hess_o = orc.hessian_pd(dog_r, orc.PD_VARIANT_REFERENCE, want_hessian=True)
        labels_o, nreg = orc.ccl(pd_r)
        regs = orc.regions(labels_r, norm_r, dog_r)
        st_r, bl_r = ref_cubin.eigen(regs["hess_f32"])
        st_o = np.empty(nreg, np.float32)
        bl_o = np.empty(nreg, np.float32)
        for i in range(nreg):
            st_o[i], bl_o[i] = orc.eigen(regs["hess_f32"][:, i])
        fin = np.isfinite(st_r) & np.isfinite(bl_r) & np.isfinite(st_o) & np.isfinite(bl_o)
        rel = lambda a, b: float(np.max(np.abs(a[fin].astype(np.float64) - b[fin]) /
                                        np.maximum(np.abs(b[fin].astype(np.float64)), 1e-30))) if fin.any() else 0.0
        rec = {
            "name": c["name"], "W": c["W"], "H": c["H"], "D": c["D"], "n_nuclei": c["n"], "seed": c["seed"],
            "synth": c["synth"], "sigma": list(c["sigma"]), "radius_norm": [c["rxy"], c["rz"]],
            "min_intensity": c["min_intensity"], "gamma": c["gamma"],
            "sha256_input": sha(vol),
            "sha256": {"norm": sha(norm_r), "dog": sha(dog_r), "hessian": sha(hess_r), "pd": sha(pd_r),
                       "labels": sha(labels_r)},
            "oracle_mismatch": {"norm": bits_equal(norm_o, norm_r), "dog_from_ref_norm": bits_equal(dog_o, dog_r),
                                "hessian_from_ref_dog": bits_equal(hess_o, hess_r),
                                "pd_from_ref_dog": bits_equal(mask_o, pd_r),
                                "labels_from_ref_pd": bits_equal(labels_o, labels_r)},
            "pd_voxels": int(pd_r.sum()), "num_regions": nreg, "ccl_iterations": iters,
            "eigen_max_rel_diff": {"structureness": rel(st_r, st_o), "blobness": rel(bl_r, bl_o)},
            "eigen_bit_mismatch": {"structureness": bits_equal(st_r, st_o), "blobness": bits_equal(bl_r, bl_o)},
            "seconds": round(time.time() - t0, 1),
        }
        result["cases"].append(rec)
        print(json.dumps(rec), flush=True)
    # -- regional erosion operator (zero border)
    vol = case_volume(CASES[0])
    er_r = ref_cubin.erosion(torch.as_tensor(vol).to(dev), 1, 1).cpu().numpy()
    er_o = orc.erosion(vol, 1, 1)
    result["erosion"] = {"case": CASES[0]["name"], "radius": [1, 1], "sha256": sha(er_r),
                         "oracle_mismatch": bits_equal(er_o, er_r)}
    with open(os.path.join(out_dir, "ref_stages.json"), "w") as f:
        json.dump(result, f, indent=1)
    print("wrote", os.path.join(out_dir, "ref_stages.json"))


def ref_pd_only(planes):
    """PositiveDefiniteKernel alone on given planes (6, D, H, W)."""
    import ctypes
    import torch
    _, D, H, W = planes.shape
    pd = torch.empty((D, H, W), dtype=torch.uint8, device=planes.device)
    ref_cubin._need(W % 8 == 0 and H % 8 == 0 and D % 8 == 0, "8^3 blocks")
    ref_cubin._launch(ref_cubin._kernel("Hessian3DFilter_element", "PositiveDefiniteKernel"),
                      (W // 8, H // 8, D // 8), (8, 8, 8),
                      [ref_cubin._p(pd), ref_cubin._p(planes), ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(D)])
    ref_cubin._sync()
    return pd


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/ref_golden.py OUT_DIR")
    main(sys.argv[1])
