"""Whole-chain parity: candidate records of the GPU path against the oracle.

Exact fields: centroid x/y/z, intensity (max mode), size, padding, record count and
order.  structureness / blobness come from region Hessian sums whose summation order
differs (double accumulation here, the reference's CUB order there): they are checked
within a relative tolerance stated below, against the oracle's sequential float sums.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest
import torch

import hdog
from helpers import params, volume, padded
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

EIGEN_RTOL = 1e-4      # structureness / blobness vs the float-sum oracle


def assert_records_match(got, ref, what, sum_intensity=False):
    assert len(got) == len(ref), "%s: %d records vs %d" % (what, len(got), len(ref))
    if len(ref) == 0:
        return
    exact = ["local_x", "local_y", "local_z", "size", "padding"] + ([] if sum_intensity else ["intensity"])
    for f in exact:
        a, b = got[f], ref[f]
        if a.dtype == np.float32:
            a, b = a.view(np.uint32), b.view(np.uint32)
        bad = np.count_nonzero(a != b)
        assert bad == 0, "%s: field %s differs in %d records" % (what, f, bad)
    tol_fields = ["structureness", "blobness"] + (["intensity"] if sum_intensity else [])
    for f in tol_fields:
        a = got[f].astype(np.float64)
        b = ref[f].astype(np.float64)
        fin = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), fin), (what, f)
        rel = np.abs(a[fin] - b[fin]) / np.maximum(np.abs(b[fin]), 1e-30)
        assert rel.max(initial=0) <= EIGEN_RTOL, (what, f, float(rel.max()))


@pytest.mark.parametrize("depth_valid", [32, 21])
def test_run_substack_matches_oracle(depth_valid):
    W, H, D = 256, 192, 32
    vol = volume(W, H, D, n_nuclei=160)
    p = params(W, H, D, margins=10)
    sub = padded(vol, D, depth_valid)
    with hdog.Context(p) as ctx:
        got = ctx.run_substack(np.ascontiguousarray(vol[:depth_valid]), depth_valid, 40)
    ref = orc.substack(orc.params_from(p), sub, depth_valid, 40)[0]
    assert len(ref) > 20
    assert_records_match(got, ref, "substack dv=%d" % depth_valid)


def test_run_substack_device_input_and_ave_mode():
    W, H, D = 160, 128, 16
    vol = volume(W, H, D, n_nuclei=60)
    p = params(W, H, D, is_ave_mode=1, sigma_z_large=1.6, extra_depth_margin=1)
    with hdog.Context(p) as ctx:
        got = ctx.run_substack(torch.from_numpy(vol).cuda(), D, 0)
    ref = orc.substack(orc.params_from(p), vol, D, 0)[0]
    assert_records_match(got, ref, "ave mode", sum_intensity=True)


@pytest.mark.parametrize("max_sub", [1, 4])
def test_run_stack_matches_substack_loop(max_sub):
    W, H, L, D = 192, 160, 100, 32
    vol = volume(W, H, L, n_nuclei=250, seed=99)
    p = params(W, H, D, margins=5)
    with hdog.Context(p, max_substacks=max_sub) as ctx:
        got = ctx.run_stack(vol)
        got_dev = ctx.run_stack(torch.from_numpy(vol).cuda())
    ref = orc.stack(orc.params_from(p), vol)
    assert len(ref) > 50
    assert_records_match(got, ref, "stack")
    assert got.tobytes() == got_dev.tobytes()


def test_run_stack_into_a_page_locked_record_array():
    """A page-locked output array receives the records straight from the device (the last
    substack of this stack is short, so it runs first and its records are appended last):
    the same records as a pageable array; one that is too small gives HDOG_ERR_CAPACITY and
    the kept result is fetched with hdog_last_records."""
    W, H, L, D = 192, 160, 100, 32
    vol = volume(W, H, L, n_nuclei=250, seed=98)
    p = params(W, H, D, margins=5)
    with hdog.Context(p, max_substacks=4) as ctx:
        ref = ctx.run_stack(vol)
        assert len(ref) > 50
        pinned = torch.empty(len(ref) * hdog.DT_LOCAL.itemsize, dtype=torch.uint8).pin_memory()
        out = pinned.numpy().view(hdog.DT_LOCAL)
        got = ctx.run_stack(vol, out=out)
        assert got.tobytes() == ref.tobytes()
        small = torch.empty((len(ref) - 1) * hdog.DT_LOCAL.itemsize, dtype=torch.uint8).pin_memory()
        n = ctypes.c_int64()
        rc = hdog.lib().hdog_run_stack(ctx._h, vol.ctypes.data, 0, L, small.data_ptr(), len(ref) - 1,
                                       ctypes.byref(n), None)
        assert rc == hdog.HDOG_ERR_CAPACITY and n.value == len(ref)
        again = np.empty(len(ref), hdog.DT_LOCAL)
        assert hdog.lib().hdog_last_records(ctx._h, again.ctypes.data, len(again), ctypes.byref(n)) == hdog.HDOG_OK
        assert again.tobytes() == ref.tobytes()
    ref_o = orc.stack(orc.params_from(p), vol)
    assert_records_match(got, ref_o, "page-locked output")


def test_hdog_main_executable_writes_reference_records(tmp_path):
    W, H, L, D = 128, 96, 40, 32
    vol = volume(W, H, L, n_nuclei=60, seed=7)
    p = params(W, H, D, margins=3)
    src = []
    for z in range(L):
        f = tmp_path / ("%06d.bin" % z)
        vol[z].tofile(f)
        src.append(str(f))
    dst = tmp_path / "out" / "100000_200000.bin"
    dst.parent.mkdir()
    dst.write_bytes(b"stale")        # removed before the first substack is appended
    pf = tmp_path / "param_gpu00.json"
    hdog.write_param_file(str(pf), p, [(str(dst), src)])
    r = subprocess.run([hdog.MAIN_PATH, str(pf)], stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 0, r.stderr.decode()
    got = np.fromfile(dst, dtype=hdog.DT_LOCAL)
    ref = orc.stack(orc.params_from(p), vol)
    assert_records_match(got, ref, "hdog_main")


def test_hdog_main_resume_metrics_and_a_short_slice(tmp_path):
    """Two stacks; one slice file holds only half a slice (its tail reads as zero, where the
    reference leaves its buffer's stale contents).  With verbose a JSON metrics line closes
    the run; no ".part" file is left; with "skip_existing" a rerun recomputes only the stack
    whose result was deleted, and gives the same file."""
    import json
    W, H, L, D = 128, 96, 40, 32
    p = params(W, H, D, margins=3)
    vols, stacks = [], []
    for k in range(2):
        vol = volume(W, H, L, n_nuclei=60, seed=70 + k)
        d = tmp_path / ("src%d" % k)
        d.mkdir()
        src = []
        for z in range(L):
            f = d / ("%06d.bin" % z)
            vol[z].tofile(f)
            src.append(str(f))
        if k == 1:   # slice 17 of stack 1: its first half only
            short = vol[17].reshape(-1)[: W * H // 2]
            short.tofile(src[17])
            vol = vol.copy()
            vol[17].reshape(-1)[W * H // 2:] = 0
        vols.append(vol)
        stacks.append((str(tmp_path / "out" / ("stack%d.bin" % k)), src))
    (tmp_path / "out").mkdir()
    pf = tmp_path / "param.json"
    hdog.write_param_file(str(pf), p, stacks)
    d = json.load(open(pf))
    d["verbose"] = True
    pf.write_text(json.dumps(d))
    r = subprocess.run([hdog.MAIN_PATH, str(pf)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    metrics = json.loads([l for l in r.stdout.splitlines() if l.startswith('{"hdog_main"')][-1])["hdog_main"]
    assert metrics["stacks_done"] == 2 and metrics["slices"] == 2 * L and metrics["status"] == 0
    assert not list((tmp_path / "out").glob("*.part"))
    first = [np.fromfile(s[0], dtype=hdog.DT_LOCAL) for s in stacks]
    for got, vol in zip(first, vols):
        assert_records_match(got, orc.stack(orc.params_from(p), vol), "hdog_main stack")
    assert metrics["records"] == sum(len(x) for x in first)
    import os
    os.remove(stacks[1][0])
    d["skip_existing"] = True
    pf.write_text(json.dumps(d))
    r = subprocess.run([hdog.MAIN_PATH, str(pf)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    metrics = json.loads([l for l in r.stdout.splitlines() if l.startswith('{"hdog_main"')][-1])["hdog_main"]
    assert metrics["stacks_done"] == 1 and metrics["stacks_skipped"] == 1
    assert np.fromfile(stacks[1][0], dtype=hdog.DT_LOCAL).tobytes() == first[1].tobytes()


def test_hdog_main_reads_ahead_in_the_serial_order(tmp_path):
    """hdog_main reads the next stack's slices while the current one runs.  Four stacks: the
    second is skipped (its result exists, skip_existing), the fourth has a missing slice
    file.  The results and the error are those of a run that reads stack after stack: the
    first and third stacks are written and equal the oracle, the skipped result is left as
    it was, the fourth stack has no result and the run exits with status 2."""
    import json
    W, H, L, D = 128, 96, 40, 32
    p = params(W, H, D, margins=3)
    (tmp_path / "out").mkdir()
    vols, stacks = [], []
    for k in range(4):
        vol = volume(W, H, L, n_nuclei=60, seed=90 + k)
        d = tmp_path / ("src%d" % k)
        d.mkdir()
        src = []
        for z in range(L):
            f = d / ("%06d.bin" % z)
            vol[z].tofile(f)
            src.append(str(f))
        vols.append(vol)
        stacks.append((str(tmp_path / "out" / ("stack%d.bin" % k)), src))
    os.remove(stacks[3][1][21])
    with open(stacks[1][0], "wb") as f:
        f.write(b"kept")
    pf = tmp_path / "param.json"
    hdog.write_param_file(str(pf), p, stacks)
    d = json.load(open(pf))
    d["verbose"] = True
    d["skip_existing"] = True
    pf.write_text(json.dumps(d))
    r = subprocess.run([hdog.MAIN_PATH, str(pf)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 2, (r.returncode, r.stderr)
    assert "000021.bin" in r.stderr
    metrics = json.loads([l for l in r.stdout.splitlines() if l.startswith('{"hdog_main"')][-1])["hdog_main"]
    assert metrics["stacks_done"] == 2 and metrics["stacks_skipped"] == 1 and metrics["status"] == hdog.HDOG_ERR_IO
    for k in (0, 2):
        got = np.fromfile(stacks[k][0], dtype=hdog.DT_LOCAL)
        assert_records_match(got, orc.stack(orc.params_from(p), vols[k]), "hdog_main stack %d" % k)
    assert open(stacks[1][0], "rb").read() == b"kept"
    assert not os.path.exists(stacks[3][0])
    assert not list((tmp_path / "out").glob("*.part"))


def test_hdog_main_write_failure_ends_the_run_in_order(tmp_path):
    """Records are written while the next stack runs; a failed write still ends the run as
    a serial run would: the second stack's result cannot be written (its directory does not
    exist), so the run exits with status 2 after the first stack's result was written, and
    the third stack's earlier result is left untouched (a serial run never reaches it)."""
    W, H, L, D = 128, 96, 40, 32
    p = params(W, H, D, margins=3)
    vols, stacks = [], []
    (tmp_path / "out").mkdir()
    for k in range(3):
        vol = volume(W, H, L, n_nuclei=60, seed=110 + k)
        d = tmp_path / ("src%d" % k)
        d.mkdir()
        src = []
        for z in range(L):
            f = d / ("%06d.bin" % z)
            vol[z].tofile(f)
            src.append(str(f))
        vols.append(vol)
        out = tmp_path / ("missing" if k == 1 else "out") / ("stack%d.bin" % k)
        stacks.append((str(out), src))
    with open(stacks[2][0], "wb") as f:
        f.write(b"earlier")
    pf = tmp_path / "param.json"
    hdog.write_param_file(str(pf), p, stacks)
    r = subprocess.run([hdog.MAIN_PATH, str(pf)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 2, (r.returncode, r.stderr)
    assert "stack1.bin.part" in r.stderr
    got = np.fromfile(stacks[0][0], dtype=hdog.DT_LOCAL)
    assert_records_match(got, orc.stack(orc.params_from(p), vols[0]), "hdog_main stack 0")
    assert open(stacks[2][0], "rb").read() == b"earlier"


def test_erosion_opt_in_pipeline():
    W, H, D = 128, 128, 16
    vol = volume(W, H, D, n_nuclei=40, seed=5)
    p = params(W, H, D, erosion_radius_xy=1, erosion_radius_z=1, sigma_z_large=1.6, extra_depth_margin=1)
    with hdog.Context(p) as ctx:
        got = ctx.run_substack(vol, D, 0)
    ref = orc.substack(orc.params_from(p), orc.erosion(vol, 1, 1), D, 0)[0]
    assert_records_match(got, ref, "eroded input")


def test_capacity_error_is_reported():
    W, H, D = 128, 128, 16
    vol = volume(W, H, D, n_nuclei=40, seed=5)
    p = params(W, H, D, sigma_z_large=1.6, extra_depth_margin=1)
    with hdog.Context(p) as ctx:
        full = ctx.run_substack(vol, D, 0)
        n = len(full)
        assert n > 2
        out = np.empty(1, hdog.DT_LOCAL)
        cnt = ctypes.c_int64()
        rc = hdog.lib().hdog_run_substack(ctx._h, vol.ctypes.data, 0, D, 0, out.ctypes.data, 1, ctypes.byref(cnt), None)
        assert rc == hdog.HDOG_ERR_CAPACITY and cnt.value == n
        # the context kept the result: fetched without running the chain again
        again = np.empty(n, hdog.DT_LOCAL)
        assert hdog.lib().hdog_last_records(ctx._h, again.ctypes.data, n, ctypes.byref(cnt)) == hdog.HDOG_OK
        assert cnt.value == n and again.tobytes() == full.tobytes()


# sigma sets: the workload's (tap radii 4, 6, 3, 5) and the reference example's (8, 12, 4,
# 5) run the radius-specialised sweep; (4, 6, 3, 3) runs the generic one.
SIGMA_SETS = {
    "workload": dict(sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2, sigma_z_large=2.4),
    "reference_example": dict(sigma_xy_small=4.0, sigma_z_small=1.8, sigma_xy_large=6.0, sigma_z_large=2.7),
    "generic": dict(sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2, sigma_z_large=1.6),
}


@pytest.mark.parametrize("sigmas", sorted(SIGMA_SETS))
@pytest.mark.parametrize("W,H,D,dv", [(68, 45, 13, 13), (256, 96, 32, 20), (132, 20, 7, 5), (64, 16, 40, 40),
                                      (184, 70, 24, 24)])
def test_fused_sweep_equals_separate_passes(W, H, D, dv, sigmas):
    vol = volume(W, H, D, n_nuclei=max(4, W * H * D // 8000), seed=W + H + D)
    p = params(W, H, D, extra_depth_margin=0, **SIGMA_SETS[sigmas])
    with hdog.Context(p) as ctx:
        fused = ctx.run_substack(np.ascontiguousarray(vol[:dv]), dv, 3)
        ctx.set_fused_sweep(False)
        plain = ctx.run_substack(np.ascontiguousarray(vol[:dv]), dv, 3)
    assert fused.tobytes() == plain.tobytes()
    ref = orc.substack(orc.params_from(p), padded(vol, D, dv), dv, 3)[0]
    assert_records_match(fused, ref, "fused %dx%dx%d %s" % (W, H, D, sigmas))


@pytest.mark.gpu
def test_run_stacks_packs_across_stacks_like_per_stack_runs():
    """hdog_run_stacks (substacks of several stacks packed into shared batches) gives each
    stack's records exactly as hdog_run_stack does, stack by stack, with the counts."""
    import torch
    W, H, D = 256, 192, 32
    p = params(W, H, D, margins=6)
    lengths = [40, 75, 9, 0, 33]
    stacks = [volume(W, H, max(L, 1), n_nuclei=max(1, L * 8), seed=9000 + i)[:L] for i, L in enumerate(lengths)]
    with hdog.Context(p, max_substacks=3) as ctx:
        per = [ctx.run_stack(np.ascontiguousarray(s)) if len(s) else np.zeros(0, hdog.DT_LOCAL) for s in stacks]
        inputs = [torch.from_numpy(np.ascontiguousarray(s)).cuda() if i % 2 == 0 else np.ascontiguousarray(s)
                  for i, s in enumerate(stacks)]
        recs, counts = ctx.run_stacks(inputs)
    assert list(counts) == [len(r) for r in per]
    assert recs.tobytes() == np.concatenate(per).tobytes()
    assert sum(len(r) for r in per) > 50
