"""HDoG cell-candidate detection throughput on GB300 (Gvox/s of unique input voxels).

Workload (one step): one camera stack, uint16 2560 x 2160 x 128, seeded synthetic:
60k nuclei (10% in touching pairs), background 100 +- 8, z attenuation 1.0 -> 0.6,
per-slice row striping +-5%.  HDoG parameters: substack depth 32, extra depth margin 3
(8 overlapping substacks per stack), DoG sigma small (xy 2.0, z 1.5), large 1.6x,
normalization radius xy 20 / z 5, min_intensity 50, margins 100, min_size 0.
A step runs normalize -> DoG -> Hessian/PD -> CCL -> features -> records for the whole
stack.  `value`: input already in HBM; `e2e`: the C-ABI call with the stack in pinned
host memory, host->device copy and record read-back inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs as one process per GPU under torch.distributed.run, each rank on its own
copy of the stack (replicas, no collective on the data path; weak scaling).
"""
import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cubic-informatics_gb300"))

METRIC = "Gvox/s HDoG→CCL→features on 1 GB300, batched vs plain; % HBM roofline"
W, H, L, DEPTH = 2560, 2160, 128, 32
PARAMS = dict(width=W, height=H, depth=DEPTH, left_margin=100, right_margin=100, top_margin=100,
              bottom_margin=100, extra_depth_margin=3, radius_norm_xy=20, radius_norm_z=5, min_intensity=50,
              gamma_n=1.0, sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2, sigma_z_large=2.4,
              min_size=0, is_ave_mode=0)
WORKLOAD = ("camera stack uint16 2560x2160x128, 60k nuclei (10% touching pairs), z-attenuation 1.0->0.6, "
            "row striping 5%; HDoG depth 32 (8 overlapping substacks), sigma_dog (2,1.5,3.2,2.4), "
            "radius_norm (20,5)")

# Compulsory bytes per processed voxel of each kernel's own inputs and outputs (each
# array read once, written once; sparse foreground-list and region traffic excluded).
# Stage totals: normalize 56 (five passes), DoG 8, Hessian + mask 5, CCL 5, features ~0.
KERNEL_BYTES_PER_VOXEL = {
    "k_mm_z": 2 + 4, "k_mm_y": 4 + 4, "k_mm_x": 4 + 8, "k_box_y": 8 + 8, "k_box_z_norm": 8 + 2 + 4,
    "k_dog_sweep": 4 + 4, "k_hess_sweep": 4 + 1, "k_dog_hess": 4 + 1, "k_conv_x": 4 + 8, "k_conv_y": 8 + 8, "k_conv_z_dog": 8 + 4,
    "k_hessian_pd": 4 + 1, "k_ccl_local": 1 + 4, "k_ccl_flatten": 1 + 0.125, "k_rank": 0.125,
    "k_accumulate": 1,
}
E2E_ALG_BYTES_PER_VOXEL = 6      # 2 B uint16 in + 4 B labels out per processed voxel
# FP32 lane operations (an FMA or an add counts one) the DoG sweep spends per output voxel
# with the workload's tap radii (xy 4 / 6, z 3 / 5): the x pass of both scales (9 + 13 taps)
# over the 16-row tile and its 12 halo rows, the y pass (9 + 13), the z pass (7 + 11), the
# difference and the scale.
DOG_FP32_LANE_OPS_PER_VOXEL = (9 + 13) * (16 + 12) / 16 + (9 + 13) + (7 + 11) + 2


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "hdog_bench_clocks_%d_rank%d.csv" % (os.getpid(), index))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


class no_gc:
    """The interpreter's cyclic garbage collector is off inside a timed region (as timeit
    does): a full collection of this process's objects takes 50-90 ms and would be charged
    to whichever call it interrupts."""

    def __enter__(self):
        gc.collect()
        gc.disable()

    def __exit__(self, *a):
        gc.enable()


def make_stack():
    from hdog import synth
    s = synth.camera_spec(depth=L)
    t = time.time()
    vol = synth.volume(s)
    return vol, time.time() - t


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def time_steps(ctx, stack, steps, warmup, stream, dist=None):
    """Device-timed steps (CUDA events on the launching stream), barrier both sides.  The
    records land in one caller-owned array reused across steps, as a long-running caller
    would keep it."""
    import torch
    import hdog
    out = np.empty(0, hdog.DT_LOCAL)
    for _ in range(warmup):
        r = ctx.run_stack(stack, stream=stream, out=out)
        if len(r) > len(out):
            out = np.empty(len(r), hdog.DT_LOCAL)
    torch.cuda.synchronize()
    ctx.timing_read()          # drop the warm-up launches from the per-kernel times
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    recs = None
    with no_gc():
        e0.record(stream)
        for _ in range(steps):
            recs = ctx.run_stack(stack, stream=stream, out=out)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if dist:
        dist.barrier()
    return ms, recs


def max_over_ranks(x, dist):
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _oracle_params():
    """The workload's parameters as the oracle's struct (no call into libhdog)."""
    from types import SimpleNamespace
    from oracle import oracle as orc
    return orc.params_from(SimpleNamespace(**PARAMS))


def _cpu_sample(vol, nsample):
    """The first `nsample` substacks of the stack's schedule, zero tail applied, and the
    unique input voxels they stand for (stack voxels x nsample / all substacks)."""
    from oracle import oracle as orc
    op = _oracle_params()
    z0s = orc.schedule(L, DEPTH, orc.depth_margin(op))
    subs = []
    for z0 in z0s[:nsample]:
        sub = np.zeros((DEPTH, H, W), np.uint16)
        dv = min(DEPTH, L - z0)
        sub[:dv] = vol[z0:z0 + dv]
        subs.append((z0, dv, sub))
    return op, subs, W * H * L * len(subs) / len(z0s), len(z0s)


def _run_cpu_sample(op, subs):
    from oracle import oracle as orc
    for z0, dv, sub in subs:
        orc.substack(op, sub, dv, z0)


def cpu_baseline(vol, steps=1, nsample=4):
    """The CPU oracle on the first `nsample` substacks of the stack's schedule: a bounded
    sample of the same workload (about 10-15 s), on every host core its OpenMP parts use."""
    op, subs, unique, nall = _cpu_sample(vol, nsample)
    t = time.time()
    for _ in range(steps):
        _run_cpu_sample(op, subs)
    dt = (time.time() - t) / steps
    return {"value": unique / dt / 1e9, "unit": "Gvox/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "the first %d of the stack's %d 2560x2160x32 substacks, %.1f s; value over the unique input "
                      "voxels they stand for (stack voxels x %d/%d); OpenMP filter passes, single-thread CCL and "
                      "region pass" % (len(subs), nall, dt, len(subs), nall)}


def run_reference(args):
    """The reference's CPU implementation of the path (the oracle port of src/3D, built
    from its C restatement; the reference's own executable needs a CUDA GPU and its host
    part cannot be built for this Arm host) on the same workload.  A step is a bounded
    sample of the stack: its first two substacks, through every stage and the records."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    vol, _ = make_stack()
    op, subs, unique, nall = _cpu_sample(vol, 2)
    for _ in range(args.warmup):
        _run_cpu_sample(op, subs)
    t = time.time()
    for _ in range(args.steps):
        _run_cpu_sample(op, subs)
    step_s = (time.time() - t) / args.steps
    value = unique / step_s / 1e9
    sample = ("each step: the first %d of the stack's %d 2560x2160x32 substacks (%.1f s); value over the unique "
              "input voxels they stand for (stack voxels x %d/%d); OpenMP filter passes, single-thread CCL and "
              "region pass" % (len(subs), nall, step_s, len(subs), nall))
    base = {"value": value, "unit": "Gvox/s", "cores": os.cpu_count(), "kind": "port", "sample": sample}
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "Gvox/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": camera_config(args.gpus), "sample": sample,
            "cpu_baseline": base,
            "e2e": {"value": value, "unit": "Gvox/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def camera_config(n_gpus):
    """The workload's description, the same for both arms."""
    nsub = 8
    return {"workload": WORKLOAD, "unique_voxels_per_step": W * H * L,
            "processed_voxels_per_step": W * H * DEPTH * nsub,
            "parallelism": "replicas" if n_gpus > 1 else "single GPU",
            "l2": "inputs larger than L2 (%.2f GB uint16 stack per step, L2 129 MB)" % (W * H * L * 2 / 1e9)}


def profile_case():
    """The small case of the ncu captures: substack 0 of the camera stack (2560 x 2160 x 32,
    177 M voxels, the workload's density of nuclei and parameters) through the whole chain,
    one warm-up run and one captured run."""
    import torch
    import hdog
    vol, _ = make_stack()
    p = hdog.make_params(**PARAMS)
    with hdog.Context(p) as ctx:
        dv = torch.from_numpy(np.ascontiguousarray(vol[:DEPTH])).cuda()
        for _ in range(2):
            r = ctx.run_substack(dv, DEPTH, 0)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "camera substack 0, 2560x2160x32", "records": int(len(r))}))
    return 0


UNEVEN_SHAPES = [(2560, 2160), (1280, 2160), (2560, 1080)]
UNEVEN_SUBSET = 6
UNEVEN_SUB = ("the first 6 stacks of the 40-stack uneven mix (z ~ U{64..512}, xy 2560x2160 / 1280x2160 / 2560x1080 "
              "with p = 1/3 each, nuclei at 2e-5 per voxel); HDoG depth 32, sigma_dog (2,1.5,3.2,2.4), "
              "radius_norm (20,5)")
UNEVEN = ("40 uneven stacks: z ~ U{64..512}, xy 2560x2160 / 1280x2160 / 2560x1080 with p = 1/3 each, "
          "nuclei at 2e-5 per voxel (the 256x256x64 case's shape and amplitude distributions); "
          "HDoG depth 32, sigma_dog (2,1.5,3.2,2.4), radius_norm (20,5)")


# The same kind of mix with small frames (a 256 x 256 tile and its two half-size edge tiles,
# nuclei at the 256 x 256 x 64 case's density): each substack is a few milliseconds of work
# or less, so the plain loop's per-substack launches and host synchronisation show.
SMALL_SHAPES = [(256, 256), (128, 256), (256, 128)]
SMALL_N = 40
SMALL_DENSITY = 400.0 / (256 * 256 * 64)
SMALL = ("40 uneven small stacks: z ~ U{64..512}, xy 256x256 / 128x256 / 256x128 with p = 1/3 each, nuclei "
         "at the 256x256x64 case's density (400 per 4.2 M voxels); HDoG depth 32, sigma_dog (2,1.5,3.2,2.4), "
         "radius_norm (20,5), margins 10")


def uneven_stacks(n, seed, dev, shapes=UNEVEN_SHAPES, density=2e-5):
    """n seeded stacks of the uneven mix on the device: z ~ U{64..512}, a frame shape each
    with p = 1/3, nuclei at `density` per voxel.  -> (list of (shape, tensor), unique voxels, s)."""
    import torch
    from hdog import synth
    rng = np.random.default_rng(seed)
    stacks, unique = [], 0
    t0 = time.time()
    for i in range(n):
        w, h = shapes[int(rng.integers(3))]
        length = int(rng.integers(64, 513))
        nn = max(1, int(round(density * w * h * length)))
        vol = synth.volume(synth.spec(w, h, length, nn, synth.SEED_BASE + 1000 + i))
        stacks.append(((w, h), torch.from_numpy(vol).to(dev)))
        unique += w * h * length
        del vol
    return stacks, unique, time.time() - t0


def run_uneven(stacks, unique, steps, warmup, max_sub, dev_id=0, params=PARAMS):
    """The batched graph form (one captured CUDA graph over all stacks, one context per frame
    shape, autotuned launch shapes) against the plain loop (one substack per launch sequence,
    stack after stack, as the reference runs them); records compared byte for byte."""
    import torch
    import hdog
    shapes = sorted({s for s, _ in stacks})
    tensors = [t for _, t in stacks]
    # plain: one context of one substack per frame shape
    plain_ctx = {k: hdog.Context(hdog.make_params(dev_id=dev_id, **dict(params, width=k[0], height=k[1])), 1)
                 for k in shapes}
    run_plain = lambda: [plain_ctx[s].run_stack(t) for s, t in stacks]
    for _ in range(1):
        prec = run_plain()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    psteps = max(1, min(steps, 2))
    with no_gc():
        a.record()
        for _ in range(psteps):
            prec = run_plain()
        b.record()
        torch.cuda.synchronize()
    pms = a.elapsed_time(b) / psteps
    for c in plain_ctx.values():
        c.close()
    prec = np.concatenate(prec)
    # graph form
    t0 = time.time()
    ctxs = [hdog.Context(hdog.make_params(dev_id=dev_id, **dict(params, width=k[0], height=k[1])), max_sub)
            for k in shapes]
    graph = hdog.Graph(ctxs, tensors)
    create_s = time.time() - t0
    for _ in range(max(1, warmup)):
        grec, counts = graph.run()
    torch.cuda.synchronize()
    with no_gc():
        a.record()
        for _ in range(steps):
            grec, counts = graph.run()
        b.record()
        torch.cuda.synchronize()
    gms = a.elapsed_time(b) / steps
    tuning = {"%dx%d" % k: c.tuning() for k, c in zip(shapes, ctxs)}
    graph.close()
    for c in ctxs:
        c.close()
    assert grec.tobytes() == prec.tobytes(), "graph and plain records differ on the uneven stacks"
    return {"value": unique / (gms * 1e-3) / 1e9, "ms_per_step": gms,
            "plain": {"value": unique / (pms * 1e-3) / 1e9, "ms_per_step": pms,
                      "mode": "one substack per launch sequence, stack after stack"},
            "batched_over_plain": pms / gms, "records_per_step": int(len(grec)),
            "mode": "one captured CUDA graph over every stack: %d substacks per context at most, persistent sweeps "
                    "over a device work queue where the autotuner chose them" % max_sub,
            "graph_create_s": round(create_s, 2), "tuning": tuning}


def uneven_workload(args):
    """The 40-stack uneven mix through the batched graph form against the plain loop.
    Stacks are generated one at a time and kept in HBM (about 79 GB)."""
    import torch
    torch.cuda.set_device(0)
    stacks, unique, gen_s = uneven_stacks(40, synth_seed(2), "cuda:0")
    res = run_uneven(stacks, unique, args.steps, args.warmup, 8)
    shapes = {}
    for s, _ in stacks:
        shapes["%dx%d" % s] = shapes.get("%dx%d" % s, 0) + 1
    line = {"metric": METRIC, "value": res["value"], "unit": "Gvox/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": UNEVEN, "stacks_per_shape": shapes, "unique_voxels_per_step": unique},
            "generator_s": round(gen_s, 1)}
    line.update({k: v for k, v in res.items() if k not in ("value", "ms_per_step")})
    print(json.dumps(line), flush=True)
    return 0


def synth_seed(k):
    from hdog import synth
    return synth.SEED_BASE + k



def stream_nuclei(w, h, d, total, seed):
    from hdog import synth
    return synth.clustered_nuclei(w, h, d, total, seed)


def run_stream(d, total_nuclei, steps, warmup, dev_id=0):
    """A dense stack of d slices (2560 x 2160) in pinned host memory, `total_nuclei` nuclei with
    30% of them in touching clusters of 2-6, through hdog_run_stack: its chunks are copied on a
    second stream while the first batches run.  Batched (8 substacks per launch) and plain (one
    per launch) forms, end to end, records compared byte for byte."""
    import torch
    import hdog
    from hdog import synth
    w, h = 2560, 2160
    t0 = time.time()
    nuc = stream_nuclei(w, h, d, total_nuclei, synth.SEED_BASE + 4)
    spec = synth.spec(w, h, d, len(nuc), synth.SEED_BASE + 4)
    host = torch.empty((d, h, w), dtype=torch.uint16).pin_memory()
    hn = host.numpy()
    for z0 in range(0, d, 128):
        hn[z0:z0 + 128] = synth.volume(spec, z0, min(d, z0 + 128), nuc=nuc)
    gen_s = time.time() - t0
    p = hdog.make_params(dev_id=dev_id, **PARAMS)
    unique = w * h * d
    res = {}
    for name, max_sub, n in (("batched", 8, steps), ("plain", 1, max(1, min(steps, 2)))):
        with hdog.Context(p, max_substacks=max_sub) as ctx:
            out = np.empty(0, hdog.DT_LOCAL)
            for _ in range(max(1, warmup)):
                r = ctx.run_stack(hn, out=out)
                if len(r) > len(out):
                    out = np.empty(len(r), hdog.DT_LOCAL)
            torch.cuda.synchronize()
            with no_gc():
                t = time.perf_counter()
                for _ in range(n):
                    r = ctx.run_stack(hn, out=out)
                torch.cuda.synchronize()
                elapsed = time.perf_counter() - t
            res[name] = (elapsed * 1e3 / n, r.copy())
            if name == "batched":   # where one more call spends its time (host phases, kernels)
                ctx.timing(True)
                ctx.timing_read()
                ctx.run_stack(hn, out=out)
                ph = ctx.timing_read()
                ctx.timing(False)
                phases = {k: round(v[1], 2) for k, v in ph.items() if k.startswith("host_")}
                phases["kernels"] = round(sum(v[1] for k, v in ph.items() if not k.startswith("host_")), 2)
    # the pinned host -> device copy rate of the whole stack on this machine
    dev = torch.empty((d, h, w), dtype=torch.uint16, device="cuda")
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    dev.copy_(host, non_blocking=True)
    b.record()
    torch.cuda.synchronize()
    h2d_gbs = unique * 2 / (a.elapsed_time(b) * 1e-3) / 1e9
    del dev
    assert res["batched"][1].tobytes() == res["plain"][1].tobytes(), "batched and plain records differ"
    bms, pms = res["batched"][0], res["plain"][0]
    nsub = len(hdog.substack_schedule(d, DEPTH, hdog.depth_margin(p)))
    return {"value": unique / (bms * 1e-3) / 1e9, "ms_per_step": bms,
            "config": {"workload": "dense stack uint16 2560x2160x%d in pinned host memory, %d nuclei, 30%% of them "
                                   "in touching clusters of 2-6; HDoG depth 32 (%d overlapping substacks), sigma_dog "
                                   "(2,1.5,3.2,2.4), radius_norm (20,5); per-substack labels as the reference"
                                   % (d, len(nuc), nsub),
                       "unique_voxels_per_step": unique, "records_per_step": int(len(res["batched"][1])),
                       "generator_s": round(gen_s, 1)},
            "mode": "end to end: pinned host stack, chunked H2D overlapping the batches, records D2H",
            "one_call_ms": phases, "pinned_h2d_gbs": round(h2d_gbs, 1),
            "plain": {"value": unique / (pms * 1e-3) / 1e9, "ms_per_step": pms, "mode": "one substack per launch"},
            "batched_over_plain": pms / bms,
            "e2e": {"value": unique / (bms * 1e-3) / 1e9, "unit": "Gvox/s", "h2d_bytes_per_step": unique * 2,
                    "d2h_bytes_per_step": int(len(res["batched"][1])) * 28}}


def stream_workload(args):
    """The 17 GB dense stack (2560 x 2160 x 1536, 1.5 M nuclei) end to end from host memory."""
    import torch
    torch.cuda.set_device(0)
    r = run_stream(1536, 1_500_000, args.steps, args.warmup)
    line = {"metric": METRIC, "value": r["value"], "unit": "Gvox/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": r["config"]}
    line.update({k: v for k, v in r.items() if k not in ("value", "ms_per_step", "config")})
    print(json.dumps(line), flush=True)
    return 0


SOFT = ("differentiable chain: 4 volumes uint16 128x512x512 (cast to float32), 3200 nuclei each; loss = mean "
        "relaxed mask score at 2000 nucleus centroids (jittered +-0.5 voxel) - mean at 2000 random voxels; "
        "gradients w.r.t. the 6 DoG sigmas, the 3 test thresholds and the input volume; radius_norm (20,5), tau 0.02")


def soft_workload(args):
    """Forward + hand-written backward of the differentiable chain on four volumes; a step
    is one loss and both gradients for every volume."""
    import torch
    import hdog
    from hdog import synth
    torch.cuda.set_device(0)
    rng = np.random.default_rng(synth.SEED_BASE + 3)
    d, h, w = 128, 512, 512
    cases = []
    for i in range(4):
        spec = synth.spec(w, h, d, 3200, synth.SEED_BASE + 300 + i)
        nuc = synth.nuclei(spec)
        vol = torch.from_numpy(synth.volume(spec, nuc=nuc).astype(np.float32)).cuda()
        c = nuc[rng.choice(len(nuc), 2000, replace=len(nuc) < 2000)][:, [2, 1, 0]] + rng.uniform(-0.5, 0.5, (2000, 3))
        lim = np.array([d - 1, h - 1, w - 1])
        pos = np.clip(np.rint(c), 0, lim).astype(np.int32)
        neg = np.stack([rng.integers(0, d, 2000), rng.integers(0, h, 2000), rng.integers(0, w, 2000)], 1).astype(np.int32)
        cases.append((vol, torch.from_numpy(pos).cuda(), torch.from_numpy(neg).cuda()))
    sig0 = [2.0, 2.0, 1.5, 3.2, 3.2, 2.4]
    kw = dict(radius_norm_xy=20, radius_norm_z=5, min_intensity=50.0, tau=0.02)

    def step(keep=True):
        out = []
        for vol, pos, neg in cases:
            v = vol.clone().requires_grad_(True)
            s = torch.tensor(sig0, dtype=torch.float32, requires_grad=True)
            b = torch.zeros(3, dtype=torch.float32, requires_grad=True)
            loss = hdog.soft.soft_loss(v, s, pos, neg, thresh=b, keep_intermediates=keep, **kw)
            loss.backward()
            out.append((float(loss.detach()), s.grad.tolist(), b.grad.tolist(), float(v.grad.abs().max())))
        return out

    def timed(keep):
        for _ in range(max(1, args.warmup)):
            step(keep)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(args.steps):
            res = step(keep)
        torch.cuda.synchronize()
        return (time.perf_counter() - t) * 1e3 / args.steps, res

    ms, res = timed(True)
    # the backward recomputing the forward chain instead (the same gradients)
    ms_re, res_re = timed(False)
    vox = 4 * d * h * w
    line = {"metric": METRIC, "value": vox / (ms * 1e-3) / 1e9, "unit": "Gvox/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": SOFT, "voxels_per_step": vox, "sigma": sig0,
                       "mode": "forward + backward per volume; the backward takes the forward chain's intermediates "
                               "from the forward's workspace"},
            "recomputed_intermediates": {"value": vox / (ms_re * 1e-3) / 1e9, "ms_per_step": ms_re,
                                         "mode": "the backward recomputes the forward chain from the input",
                                         "same_losses": all(a[0] == r[0] for a, r in zip(res, res_re)),
                                         "max_rel_diff_sigma_gradients": max(
                                             abs(x - y) / max(abs(y), 1e-30)
                                             for a, r in zip(res, res_re) for x, y in zip(a[1], r[1]))},
            "volumes": [{"loss": r[0], "grad_sigma": r[1], "grad_thresh": r[2], "max_abs_grad_volume": r[3]}
                        for r in res],
            "checks": "gradients checked against an FP64 reference and FP64 central differences in tests/test_soft.py "
                      "(a 14x40x44 volume, also at this workload's normalization reach and at 40, and a 24x72x80 "
                      "crop of a 128x512x512 volume of this workload)"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-stack subset of the default line")
    ap.add_argument("--no-stream", action="store_true", help="skip the dense-stack subset of the default line")
    ap.add_argument("--workload", default="camera", choices=["camera", "uneven", "stream", "soft"],
                    help="camera: the 2560x2160x128 stack (default); uneven: the 40-stack mix; "
                         "stream: the 17 GB stack from host memory; soft: the differentiable chain")
    ap.add_argument("--profile-case", action="store_true",
                    help="run substack 0 of the camera stack twice (the small case the ncu summaries capture)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return profile_case()
    if args.workload == "uneven":
        return uneven_workload(args)
    if args.workload == "stream":
        return stream_workload(args)
    if args.workload == "soft":
        return soft_workload(args)

    import torch
    import hdog
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    hdog.lib()
    vol, gen_s = make_stack()
    stream = torch.cuda.current_stream()
    p = hdog.make_params(dev_id=local, **PARAMS)
    margin = hdog.depth_margin(p)
    nsub = len(hdog.substack_schedule(L, DEPTH, margin))
    unique = W * H * L
    processed = W * H * DEPTH * nsub
    assert processed == camera_config(ws)["processed_voxels_per_step"]

    stack_dev = torch.from_numpy(vol).to(dev)
    host = torch.from_numpy(vol).pin_memory()
    host_np = host.numpy()

    batched = hdog.Context(p, max_substacks=nsub)
    # ---- batched, device-resident input (the headline `value`)
    batched.timing(True)
    clocks = ClockSampler(local)
    with clocks:
        ms, recs = time_steps(batched, stack_dev, args.steps, args.warmup, stream, dist)
    kt_all = batched.timing_read()
    batched.timing(False)
    ktimes = {k: v for k, v in kt_all.items() if not k.startswith("host_")}
    host_phases = {k: round(v[1] / args.steps, 3) for k, v in kt_all.items() if k.startswith("host_")}
    ms = max_over_ranks(ms, dist)
    ms_step = ms / args.steps
    value = unique * ws / (ms_step * 1e-3) / 1e9
    n_records = len(recs)

    # ---- end to end through the C ABI: pinned host stack, H2D + records D2H inside
    # the caller's record array in page-locked memory, as its stack is: the library then
    # copies the records straight into it
    e2e_pinned = torch.empty(n_records * hdog.DT_LOCAL.itemsize, dtype=torch.uint8).pin_memory()
    e2e_out = e2e_pinned.numpy().view(hdog.DT_LOCAL)
    for _ in range(args.warmup):
        batched.run_stack(host_np, out=e2e_out)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    call_ms = []
    with no_gc():
        t0 = time.perf_counter()
        for _ in range(args.steps):
            tc = time.perf_counter()
            recs_e2e = batched.run_stack(host_np, out=e2e_out)   # returns after its records are in e2e_out
            call_ms.append((time.perf_counter() - tc) * 1e3)
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3
    e2e_ms = max_over_ranks(e2e_ms, dist) / args.steps
    assert recs_e2e.tobytes() == recs.tobytes(), "host-input run differs from device-input run"
    # where an end-to-end call spends its time (one more call, outside the timed loop, with
    # kernel and host-phase timing on)
    batched.timing(True)
    batched.timing_read()
    batched.run_stack(host_np, out=e2e_out)
    e2e_phases = {k: round(v[1], 3) for k, v in batched.timing_read().items()}
    # six more timed calls, each with its host phases, to show where a slow call spends its time
    diag = []
    for _ in range(6):
        batched.timing_read()
        tc = time.perf_counter()
        batched.run_stack(host_np, out=e2e_out)
        ph = batched.timing_read()
        diag.append({"call_ms": round((time.perf_counter() - tc) * 1e3, 2),
                     **{k: round(v[1], 2) for k, v in ph.items() if k.startswith("host_")}})
    batched.timing(False)
    e2e_kernel_ms = round(sum(v for k, v in e2e_phases.items() if not k.startswith("host_")), 3)
    # the pinned host -> device copy rate of this machine, for reading the end-to-end figure
    h2d_ms = []
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        stack_dev.copy_(host, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        h2d_ms.append(a.elapsed_time(b))
    h2d_gbs = unique * 2 / (min(h2d_ms) * 1e-3) / 1e9

    # ---- plain: one substack per launch sequence (the reference's processing order)
    plain = hdog.Context(p, max_substacks=1)
    plain_steps = max(1, min(args.steps, 3))
    pms, precs = time_steps(plain, stack_dev, plain_steps, 1, stream, dist)
    pms = max_over_ranks(pms, dist) / plain_steps
    assert precs.tobytes() == recs.tobytes(), "plain and batched records differ"
    plain_value = unique * ws / (pms * 1e-3) / 1e9
    batched.close()
    plain.close()

    # ---- roofline of the dominant kernel (live CUDA-event times from the timed region)
    peak, peak_kind = peaks()
    launches = sum(c for c, _ in ktimes.values())
    dense = {k: v for k, v in ktimes.items() if k in KERNEL_BYTES_PER_VOXEL} or ktimes
    top = max(dense.items(), key=lambda kv: kv[1][1])
    kname, (kcount, ktotal) = top
    per_launch_voxels = processed      # one launch covers every substack of the step
    alg = KERNEL_BYTES_PER_VOXEL.get(kname, 0) * per_launch_voxels
    avg_ms = ktotal / kcount
    achieved = alg / (avg_ms * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tp):
        t = json.load(open(tp))
        if kname in t.get("bytes_per_voxel", {}):
            traffic = t["bytes_per_voxel"][kname] * per_launch_voxels
    e2e_alg_gbs = E2E_ALG_BYTES_PER_VOXEL * processed / (ms_step * 1e-3) / 1e9
    # the DoG sweep against the FP32 pipe: its FMA chains are fixed by the reference's
    # rounding, so the kernel is bound by FP32 issue, not by its 8 bytes per voxel
    fp32 = None
    clk = clocks.summary()
    if "k_dog_sweep" in ktimes and clk:
        cnt, tot = ktimes["k_dog_sweep"]
        ops = DOG_FP32_LANE_OPS_PER_VOXEL * processed
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        peak_ops = 128 * sms * clk["sm_mhz"] * 1e6
        fp32 = {"kernel": "k_dog_sweep", "lane_ops_per_voxel": DOG_FP32_LANE_OPS_PER_VOXEL,
                "achieved_tops": ops / (tot / cnt * 1e-3) / 1e12, "peak_tops": peak_ops / 1e12,
                "frac": ops / (tot / cnt * 1e-3) / peak_ops,
                "peak_source": "nominal: 128 FP32 lanes per SM x %d SMs x %.0f MHz sampled" % (sms, clk["sm_mhz"])}

    line = {
        "metric": METRIC, "value": value, "unit": "Gvox/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": camera_config(ws),
        "mode": "batched: %d substacks per launch" % nsub, "records_per_step": n_records,
        "generator_s": round(gen_s, 1),
        "plain": {"value": plain_value, "ms_per_step": pms, "mode": "one substack per launch sequence"},
        "batched_over_plain": value / plain_value,
        "e2e": {"value": unique * ws / (e2e_ms * 1e-3) / 1e9, "unit": "Gvox/s",
                "h2d_bytes_per_step": unique * 2, "d2h_bytes_per_step": n_records * 28,
                "ms_per_step": e2e_ms, "pinned_h2d_gbs": round(h2d_gbs, 1),
                "call_ms": {"median": round(statistics.median(call_ms), 2), "min": round(min(call_ms), 2),
                            "max": round(max(call_ms), 2), "all": [round(x, 2) for x in call_ms]},
                "one_call": {"kernel_ms": e2e_kernel_ms,
                             "host_ms": {k: v for k, v in e2e_phases.items() if k.startswith("host_")}},
                "phased_calls": diag},
        "gpu_launches": int(launches),
        "kernel_ms_per_step": {k: round(v[1] / args.steps, 4) for k, v in sorted(ktimes.items(), key=lambda kv: -kv[1][1])},
        "host_ms_per_step": host_phases,
        # algorithmic GB/s of each dense kernel (its per-voxel bytes over its event time)
        "kernel_alg_gbs": {k: round(KERNEL_BYTES_PER_VOXEL[k] * processed * v[0] / (v[1] * 1e-3) / 1e9, 1)
                           for k, v in ktimes.items() if k in KERNEL_BYTES_PER_VOXEL and v[1] > 0},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "alg_bytes_per_launch": alg, "avg_launch_ms": avg_ms,
                     "end_to_end_alg_gbs": e2e_alg_gbs, "end_to_end_frac": e2e_alg_gbs / peak,
                     "fp32_pipe": fp32},
        "clocks": clk,
    }
    if not args.no_uneven:
        # the uneven-stack subset: the batched graph form against the plain loop
        del stack_dev
        torch.cuda.empty_cache()
        ustacks, uunique, ugen = uneven_stacks(UNEVEN_SUBSET, synth_seed(2), dev)
        u = run_uneven(ustacks, uunique, max(2, min(args.steps, 4)), 1, 8, local)
        u["config"] = {"workload": UNEVEN_SUB, "unique_voxels_per_step": uunique,
                       "frames": sorted({"%dx%d" % sh for sh, _ in ustacks}), "generator_s": round(ugen, 1)}
        u["value"] = u["value"] * ws
        u["plain"]["value"] = u["plain"]["value"] * ws
        line["uneven"] = u
        del ustacks
        # the same forms on small frames, where per-substack launch and host costs matter
        sstacks, sunique, sgen = uneven_stacks(SMALL_N, synth_seed(5), dev, SMALL_SHAPES, SMALL_DENSITY)
        small_params = dict(PARAMS, left_margin=10, right_margin=10, top_margin=10, bottom_margin=10)
        su = run_uneven(sstacks, sunique, max(3, min(args.steps, 5)), 2, 64, local, small_params)
        su["config"] = {"workload": SMALL, "unique_voxels_per_step": sunique,
                        "frames": sorted({"%dx%d" % sh for sh, _ in sstacks}), "generator_s": round(sgen, 1)}
        su["value"] = su["value"] * ws
        su["plain"]["value"] = su["plain"]["value"] * ws
        line["uneven_small"] = su
        del sstacks
    if not args.no_stream:
        # the dense streaming stack at a quarter of its depth (384 slices, the same density of
        # nuclei and clusters), end to end from host memory, batched against plain
        torch.cuda.empty_cache()
        line["stream"] = run_stream(384, 375_000, max(2, min(args.steps, 3)), 1, local)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(vol)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
