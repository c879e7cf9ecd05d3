"""The batched graph form (hdog_graph_*) and the autotuner on uneven stacks.

Stacks of uneven depth in three frame shapes run through one captured CUDA graph; the
records must equal, byte for byte, the plain per-stack calls (hdog_run_stack, one substack
per launch), stack by stack in the caller's order, and the per-stack counts must add up.
The first stack of each shape is also checked against the CPU oracle.  A stack whose mask
overflows the foreground list inside the graph makes the run fall back to the per-stack
path, with the same records.
"""
import numpy as np
import pytest
import torch

import hdog
from helpers import params, volume
from oracle import oracle as orc
from test_gpu_pipeline import assert_records_match
from test_zz_overflow_paths import spot_lattice

pytestmark = pytest.mark.gpu

SHAPES = [(256, 192), (128, 192), (256, 96)]


def _stacks(seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(7):
        w, h = SHAPES[i % 3]
        length = int(rng.integers(20, 90))
        out.append(volume(w, h, length, seed=1000 + i))
    return out


def _plain(p_of, vols):
    recs, counts = [], []
    for v in vols:
        D, H, W = v.shape
        with hdog.Context(p_of(W, H), max_substacks=1) as ctx:
            r = ctx.run_stack(torch.from_numpy(v).cuda())
        recs.append(r)
        counts.append(len(r))
    return np.concatenate(recs), np.array(counts)


def _p(W, H):
    return params(W, H, 32, margins=4)


def test_graph_equals_per_stack_calls_and_oracle():
    vols = _stacks()
    ref, ref_counts = _plain(_p, vols)
    ctxs = [hdog.Context(_p(w, h), max_substacks=4) for w, h in SHAPES]
    dev = [torch.from_numpy(v).cuda() for v in vols]
    with hdog.Graph(ctxs, dev) as g:
        for _ in range(2):   # a graph launches any number of times
            got, counts = g.run()
            assert np.array_equal(counts, ref_counts)
            assert got.tobytes() == ref.tobytes()
    for c in ctxs:
        t = c.tuning()
        assert t["batch"] >= 1 and t["dog_per_sm"] in (0, 2, 3) and t["hess_per_sm"] in (0, 4, 5), t
        c.close()
    # the first stack of each shape against the oracle
    off = np.concatenate([[0], np.cumsum(ref_counts)])
    for i in range(3):
        D, H, W = vols[i].shape
        want = orc.stack(orc.params_from(_p(W, H)), vols[i])
        assert_records_match(got[off[i]:off[i + 1]], want, "graph stack %d" % i)


def test_graph_falls_back_when_a_batch_overflows():
    W, H = 128, 96
    p = params(W, H, 32, extra_depth_margin=0, sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2,
               sigma_z_large=2.4)
    vols = [volume(W, H, 40, seed=77), spot_lattice(W, H, 48, 14, 5.5), volume(W, H, 60, seed=78)]
    ref, ref_counts = _plain(lambda w, h: p, vols)
    with hdog.Context(p, max_substacks=2) as ctx:
        with hdog.Graph([ctx], [torch.from_numpy(v).cuda() for v in vols]) as g:
            got, counts = g.run()
    assert np.array_equal(counts, ref_counts)
    assert got.tobytes() == ref.tobytes()


def test_autotune_reports_its_choice():
    W, H, L = 256, 192, 80
    v = torch.from_numpy(volume(W, H, L, seed=5)).cuda()
    with hdog.Context(_p(W, H), max_substacks=4) as ctx:
        t = ctx.autotune(v)
        assert set(("k_dog_sweep_ms", "k_hess_sweep_ms", "dog_per_sm", "hess_per_sm", "batch")) <= set(t)
        assert all(x > 0 for x in t["k_hess_sweep_ms"])
        # the tuned launch shapes give the same records as the defaults of a fresh context
        a = ctx.run_stack(v)
    with hdog.Context(_p(W, H), max_substacks=1) as plain:
        b = plain.run_stack(v)
    assert a.tobytes() == b.tobytes()


def test_graph_with_contexts_of_more_substacks_than_one_descriptor_launch_holds():
    """Contexts of 40 substacks (the batch descriptors then take three launches of 16): the
    graph's records equal the per-stack calls' on many short stacks of small frames, where
    a batch spans several stacks."""
    rng = np.random.default_rng(21)
    vols = []
    for i in range(12):
        w, h = SHAPES[i % 3]
        vols.append(volume(w // 2, h // 2, int(rng.integers(40, 160)), seed=2000 + i))
    shapes = sorted({(v.shape[2], v.shape[1]) for v in vols})
    ref, ref_counts = _plain(_p, vols)
    assert ref_counts.sum() > 50
    ctxs = [hdog.Context(_p(w, h), max_substacks=40) for w, h in shapes]
    with hdog.Graph(ctxs, [torch.from_numpy(v).cuda() for v in vols]) as g:
        for _ in range(2):
            got, counts = g.run()
            assert np.array_equal(counts, ref_counts)
            assert got.tobytes() == ref.tobytes()
    for c in ctxs:
        c.close()
