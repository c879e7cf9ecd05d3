"""Shared test cases: parameters and seeded volumes of the HDoG path."""
import numpy as np

import hdog
from hdog import synth
from oracle import oracle as orc

# DoG sigma_small = (xy 2.0, z 1.5), sigma_large = 1.6 x; normalization radius xy 20, z 5.
CFG_PARAMS = dict(sigma_xy_small=2.0, sigma_z_small=1.5, sigma_xy_large=3.2, sigma_z_large=2.4,
                  radius_norm_xy=20, radius_norm_z=5, gamma_n=1.0, min_intensity=50, min_size=0,
                  extra_depth_margin=3, is_ave_mode=0)


def params(W, H, D, margins=0, **kw):
    d = dict(CFG_PARAMS)
    d.update(width=W, height=H, depth=D, left_margin=margins, right_margin=margins, top_margin=margins,
             bottom_margin=margins)
    d.update(kw)
    return hdog.make_params(**d)


def volume(W, H, D, n_nuclei=None, seed=synth.SEED_BASE + 7, **kw):
    if n_nuclei is None:
        n_nuclei = max(1, int(W * H * D / 10500))
    s = synth.spec(W, H, D, n_nuclei, seed, **kw)
    return synth.volume(s)


def padded(vol, D, depth_valid):
    sub = np.zeros((D,) + vol.shape[1:], np.uint16)
    sub[:depth_valid] = vol[:depth_valid]
    return sub


def oracle_params(p):
    return orc.params_from(p)


def rel_close(a, b, rtol, atol=0.0):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.all(np.abs(a - b) <= atol + rtol * np.maximum(np.abs(a), np.abs(b)))
