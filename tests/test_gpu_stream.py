"""The dense streaming stack in small: a stack in pinned host memory, 30% of its nuclei in
touching clusters of 2-6 (many of them across the overlapping substacks' boundaries), through
hdog_run_stack with its chunked copy, in batches of several substacks and one substack at a
time.  Both must give the oracle's records (each substack labelled on its own, as the
reference does), byte for byte between the two forms."""
import numpy as np
import pytest
import torch

import hdog
from hdog import synth
from helpers import params
from oracle import oracle as orc
from test_gpu_pipeline import assert_records_match

pytestmark = pytest.mark.gpu


def test_clustered_stack_from_host_memory_matches_the_oracle():
    W, H, L = 640, 720, 100
    total = int(W * H * L * 1.5e6 / (2560 * 2160 * 1536))    # the streaming stack's density
    nuc = synth.clustered_nuclei(W, H, L, total, synth.SEED_BASE + 44)
    s = synth.spec(W, H, L, len(nuc), synth.SEED_BASE + 44)
    vol = synth.volume(s, nuc=nuc)
    host = torch.from_numpy(vol).pin_memory()
    p = params(W, H, 32, margins=10)
    op = orc.params_from(p)
    sched = orc.schedule(L, p.depth, orc.depth_margin(op))
    assert len(sched) >= 5
    got = {}
    for max_sub in (4, 1):
        with hdog.Context(p, max_substacks=max_sub) as ctx:
            got[max_sub] = ctx.run_stack(host.numpy())
    assert got[4].tobytes() == got[1].tobytes()
    want = orc.stack(op, vol)
    assert len(want) > 1000
    assert_records_match(got[4], want, "clustered stack from host memory")
