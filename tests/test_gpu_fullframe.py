"""Full camera-frame checks (2560 x 2160): the sizes where races in the normalization tiles
or the labelling would show.  The normalized volume, DoG and labels of a 2560x2160x32
substack equal the oracle's; the whole 128-slice stack gives byte-identical records run
after run, from device or host input, batched or one substack at a time."""
import numpy as np
import pytest
import torch

import hdog
from hdog import synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

W, H = 2560, 2160
P = dict(width=W, height=H, depth=32, left_margin=100, right_margin=100, top_margin=100, bottom_margin=100,
         extra_depth_margin=3, radius_norm_xy=20, radius_norm_z=5, min_intensity=50, gamma_n=1.0,
         sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2, sigma_z_large=2.4, min_size=0, is_ave_mode=0)


@pytest.fixture(scope="module")
def stack():
    return synth.volume(synth.camera_spec(depth=128))


def test_fullframe_substack_stages_match_oracle(stack):
    p = hdog.make_params(**P)
    sub = np.ascontiguousarray(stack[:32])
    with hdog.Context(p) as ctx:
        img = torch.from_numpy(sub).cuda()
        norm = ctx.normalize(img)
        dog = ctx.dog(norm)
        mask, _ = ctx.hessian_pd(dog)
        labels = ctx.ccl(mask)
        g = [t.cpu().numpy() for t in (norm, dog, mask, labels)]
    # normalized volume and DoG of the full frame, bit for bit against the oracle's
    o_norm = orc.normalize(sub, P["radius_norm_xy"], P["radius_norm_z"], float(P["min_intensity"]))
    bad = np.count_nonzero(o_norm.view(np.uint32) != g[0].view(np.uint32))
    assert bad == 0, "normalized volume: %d of %d values differ" % (bad, o_norm.size)
    o_dog = orc.dog(o_norm, P["sigma_xy_small"], P["sigma_z_small"], P["sigma_xy_large"], P["sigma_z_large"],
                    P["gamma_n"])
    bad = np.count_nonzero(o_dog.view(np.uint32) != g[1].view(np.uint32))
    assert bad == 0, "DoG: %d of %d values differ" % (bad, o_dog.size)
    o_mask, _ = orc.hessian_pd(g[1])
    assert np.array_equal(o_mask, g[2])
    o_labels, n = orc.ccl(g[2])
    bad = np.count_nonzero(o_labels != g[3])
    assert bad == 0, "%d of %d labels differ" % (bad, o_labels.size)
    assert n > 100000


def test_fullframe_stack_records_are_deterministic(stack):
    p = hdog.make_params(**P)
    dev = torch.from_numpy(stack).cuda()
    with hdog.Context(p, max_substacks=8) as ctx:
        a = ctx.run_stack(dev)
        b = ctx.run_stack(dev)
        c = ctx.run_stack(np.ascontiguousarray(stack))
    with hdog.Context(p, max_substacks=1) as ctx:
        d = ctx.run_stack(dev)
    assert len(a) > 100000
    assert a.tobytes() == b.tobytes()
    assert a.tobytes() == c.tobytes()
    assert a.tobytes() == d.tobytes()


def test_fullframe_stack_records_match_oracle(stack):
    """The whole 2560x2160x128 stack (8 substacks, ~1.3M records) against the oracle:
    exact centroids, intensity and size; eigen features within 1e-4 relative."""
    from test_gpu_pipeline import assert_records_match
    p = hdog.make_params(**P)
    with hdog.Context(p, max_substacks=8) as ctx:
        got = ctx.run_stack(torch.from_numpy(stack).cuda())
    ref = orc.stack(orc.params_from(p), stack)
    assert len(ref) > 1000000
    assert_records_match(got, ref, "camera stack")


def test_fullframe_depth64_substacks_match_oracle(stack):
    """Substacks of depth 64 at the full frame (353.9 M voxels each, the largest the
    reference's 32-bit plane offsets allow at 2560 x 2160): the stack's three substacks,
    batched, against the oracle."""
    from test_gpu_pipeline import assert_records_match
    p = hdog.make_params(**dict(P, depth=64))
    with hdog.Context(p, max_substacks=3) as ctx:
        got = ctx.run_stack(torch.from_numpy(stack).cuda())
    op = orc.params_from(p)
    assert len(orc.schedule(stack.shape[0], 64, orc.depth_margin(op))) == 3
    ref = orc.stack(op, stack)
    assert len(ref) > 500000
    assert_records_match(got, ref, "camera stack, depth 64")
