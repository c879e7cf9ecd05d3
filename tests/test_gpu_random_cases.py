"""Seeded random cases of the whole chain against the oracle.

Each case draws a frame (3 to 200 voxels wide, 2 to 150 high: widths that are and are not
multiples of 4 and 16, so the radius-specialised sweeps, the generic fused sweep and the
separate passes all run), a stack length (1 to 90 slices, within a voxel budget that keeps
the oracle to a fraction of a second), a substack depth above twice the depth margin, DoG
sigmas of the specialised radii and of others, normalization radii from 0 to 25 in xy and
0 to 6 in z, the intensity threshold, margins, the minimum size, both intensity modes and
the context's batch size.  The records must equal the oracle's: record count and order,
centroids, size and (max mode) intensity bit for bit, the eigen features within
EIGEN_RTOL (the region sums' association differs, see test_gpu_pipeline).
"""
import numpy as np
import pytest

import hdog
from helpers import params, volume
from oracle import oracle as orc
from test_gpu_pipeline import assert_records_match

pytestmark = pytest.mark.gpu

CASES = 24
VOXEL_BUDGET = 350_000
# (xy small, z small, xy large, z large): the two radius-specialised sets, then others
SIGMAS = [(2.0, 1.5, 3.2, 2.4), (4.0, 1.8, 6.0, 2.7), (1.0, 1.0, 1.6, 1.6), (1.5, 0.8, 2.4, 1.3),
          (2.5, 1.2, 3.0, 2.0)]


def draw(k):
    rng = np.random.default_rng(90_000 + k)
    W = int(rng.integers(3, 201))
    H = int(rng.integers(2, 151))
    L = int(min(rng.integers(1, 91), max(1, VOXEL_BUDGET // (W * H))))
    sxy, sz, lxy, lz = SIGMAS[int(rng.integers(len(SIGMAS)))]
    extra = int(rng.integers(0, 4))
    margin = int(hdog.gaussian_taps(lz)[1]) + extra
    D = int(rng.choice([d for d in (8, 16, 24, 32, 40) if d > 2 * margin]))
    kw = dict(sigma_xy_small=sxy, sigma_z_small=sz, sigma_xy_large=lxy, sigma_z_large=lz,
              radius_norm_xy=int(rng.integers(0, 26)), radius_norm_z=int(rng.integers(0, 7)),
              min_intensity=int(rng.choice([0, 50, 120])), extra_depth_margin=extra,
              min_size=int(rng.choice([0, 3])), is_ave_mode=int(rng.integers(0, 2)))
    margins = int(rng.integers(0, 6))
    max_sub = int(rng.integers(1, 5))
    n_nuclei = max(1, W * H * L // 3000)
    return W, H, L, D, margins, max_sub, n_nuclei, kw


@pytest.mark.parametrize("k", range(CASES))
def test_random_case_matches_the_oracle(k):
    W, H, L, D, margins, max_sub, n_nuclei, kw = draw(k)
    vol = volume(W, H, L, n_nuclei=n_nuclei, seed=91_000 + k)
    p = params(W, H, D, margins=margins, **kw)
    with hdog.Context(p, max_substacks=max_sub) as ctx:
        got = ctx.run_stack(vol)
    ref = orc.stack(orc.params_from(p), vol)
    what = "case %d: %dx%dx%d depth %d, %s, margins %d, %d per batch" % (k, W, H, L, D, kw, margins, max_sub)
    assert_records_match(got, ref, what, sum_intensity=bool(kw["is_ave_mode"]))


def test_the_cases_cover_both_sweep_forms_and_the_separate_passes():
    """The premise of the cases above: they include widths that are multiples of 4 (fused
    sweeps) and that are not (separate passes), both specialised sigma sets and others, and
    the copy path of the normalization (a radius of 0)."""
    drawn = [draw(k) for k in range(CASES)]
    assert any(c[0] % 4 == 0 for c in drawn) and any(c[0] % 4 != 0 for c in drawn)
    sig = {(c[7]["sigma_xy_small"], c[7]["sigma_z_small"]) for c in drawn}
    assert (2.0, 1.5) in sig and (4.0, 1.8) in sig and len(sig) >= 4
    assert any(c[7]["radius_norm_xy"] == 0 or c[7]["radius_norm_z"] == 0 for c in drawn)
    assert any(c[7]["is_ave_mode"] for c in drawn) and not all(c[7]["is_ave_mode"] for c in drawn)
