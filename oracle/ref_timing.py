"""TEST INFRASTRUCTURE: times the reference's own CUDA kernels (the GPU baseline).

Runs the unmodified CUBIC-informatics src/3D kernels (sm_103a cubins built by
oracle/build_oracle.py, launched by oracle/ref_cubin.py with the reference's grid
shapes and host-side loop structure) on one 2560 x 2160 x 32 substack of the seeded
camera stack, and prints one JSON line with the CUDA-event time of each stage:

    python oracle/ref_timing.py [--reps 3]

Stages: Normalize3DFilter (NormalizeFilter.cu:603-654), DoG3DFilter
(DoG3DFilter.cu:417-437), HessianPositiveDefiniteWithElement
(Hessian3DFilter_element.cu:355-388), CCL (CCL3D.cu:81-117, with its host round trips
per iteration).  The regional features (RegionalFeatures.cu: 10 CUB radix sorts of N
key/value pairs plus reduce-by-key) have no cubin-level launcher here and are NOT
included, so the reference's whole-chain time is this sum plus those sorts.
"""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cubic-informatics_gb300"))

from oracle import oracle as orc  # noqa: E402
from oracle import ref_cubin  # noqa: E402
from hdog import synth  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    import torch
    if not ref_cubin.available():
        print(json.dumps({"unavailable": "reference cubins not built (oracle/_ref)"}))
        return 0
    W, H, D = 2560, 2160, 32
    sig = (2.0, 1.5, 3.2, 2.4)
    vol = synth.volume(synth.camera_spec(depth=D))
    img = torch.as_tensor(vol).to(torch.device("cuda:0"))
    normalizer = orc.dog_normalizer(sig[0], sig[1], 1.0)

    def stage(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out = fn()
        b.record()
        torch.cuda.synchronize()
        return out, a.elapsed_time(b)

    times = {"normalize": [], "dog": [], "hessian_pd": [], "ccl": []}
    iters = None
    for _ in range(args.reps + 1):   # the first pass loads the modules and warms up
        norm, t1 = stage(lambda: ref_cubin.normalize(img, 20, 5, 50.0))
        dog, t2 = stage(lambda: ref_cubin.dog(norm, sig, orc.gauss_taps, normalizer))
        (hess, pd), t3 = stage(lambda: ref_cubin.hessian_pd(dog))
        (labels, iters), t4 = stage(lambda: ref_cubin.ccl(pd))
        for k, t in zip(times, (t1, t2, t3, t4)):
            times[k].append(t)
        del hess, labels
    med = {k: sorted(v[1:])[len(v[1:]) // 2] for k, v in times.items()}
    total = sum(med.values())
    vox = W * H * D
    print(json.dumps({"reference_gpu_stages_ms": {k: round(v, 3) for k, v in med.items()},
                      "sum_ms": round(total, 3), "voxels": vox, "ccl_iterations": iters,
                      "gvox_per_s_processed": vox / (total * 1e-3) / 1e9,
                      "case": "2560x2160x32 camera substack, sigma (2,1.5,3.2,2.4), radius_norm (20,5)",
                      "excluded": "regional features (CUB sorts), host I/O",
                      "gpu": torch.cuda.get_device_name(0)}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
