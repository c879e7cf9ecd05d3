"""Seeded synthetic volumes (ctypes over libhdog_synth.so, csrc/synth.c).

The benchmark configurations of the HDoG path, written out with their parameters:
  cube   : uint16 64 x 256 x 256, 400 nuclei >= 8 voxels apart, background 100 +- 8
  camera : uint16 128 x 2160 x 2560, 60k nuclei, 10% in touching pairs, z attenuation
           1.0 -> 0.6 and per-slice row striping +-5%
Nuclei: sigma_xy ~ U[2, 3.5], sigma_z ~ U[1.2, 2] voxels, peak ~ U[300, 3000].
"""
import ctypes
import os

import numpy as np

from . import SYNTH_PATH, HDoGError, HDOG_ERR_ARG

SEED_BASE = 20261203


class synth_spec(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int), ("depth", ctypes.c_int), ("n_nuclei", ctypes.c_int),
        ("seed", ctypes.c_uint64),
        ("bg_mean", ctypes.c_double), ("bg_sd", ctypes.c_double),
        ("sigma_xy_lo", ctypes.c_double), ("sigma_xy_hi", ctypes.c_double),
        ("sigma_z_lo", ctypes.c_double), ("sigma_z_hi", ctypes.c_double),
        ("peak_lo", ctypes.c_double), ("peak_hi", ctypes.c_double),
        ("min_separation", ctypes.c_double), ("pair_fraction", ctypes.c_double),
        ("pair_distance_factor", ctypes.c_double), ("atten_z_end", ctypes.c_double),
        ("stripe_amplitude", ctypes.c_double),
    ]


class nucleus(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("x", "y", "z", "sigma_xy", "sigma_z", "peak")]


_lib = None


def _L():
    global _lib
    if _lib is None:
        if not os.path.exists(SYNTH_PATH):
            raise HDoGError(HDOG_ERR_ARG, "libhdog_synth.so is not built; run hdog.build()")
        L = ctypes.CDLL(SYNTH_PATH)
        L.hdog_synth_default_spec.argtypes = [ctypes.POINTER(synth_spec), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_uint64]
        L.hdog_synth_nuclei.restype = ctypes.c_int64
        L.hdog_synth_nuclei.argtypes = [ctypes.POINTER(synth_spec), ctypes.c_void_p, ctypes.c_int64]
        L.hdog_synth_render.restype = ctypes.c_int
        L.hdog_synth_render.argtypes = [ctypes.POINTER(synth_spec), ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p]
        _lib = L
    return _lib


def spec(width, height, depth, n_nuclei, seed, **kw):
    s = synth_spec()
    _L().hdog_synth_default_spec(ctypes.byref(s), width, height, depth, n_nuclei, seed)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def cube_spec(seed=SEED_BASE + 0):
    return spec(256, 256, 64, 400, seed)


def camera_spec(depth=128, seed=SEED_BASE + 1, n_nuclei=60000):
    return spec(2560, 2160, depth, n_nuclei, seed, pair_fraction=0.1, atten_z_end=0.6, stripe_amplitude=0.05)


def nuclei(s):
    buf = (nucleus * max(1, s.n_nuclei))()
    n = _L().hdog_synth_nuclei(ctypes.byref(s), ctypes.cast(buf, ctypes.c_void_p), s.n_nuclei)
    if n < 0:
        raise HDoGError(HDOG_ERR_ARG, "bad synthetic spec")
    arr = np.ctypeslib.as_array(buf)[:n]
    return arr.view(np.float64).reshape(-1, 6).copy() if n else np.zeros((0, 6))


def volume(s, z_begin=0, z_end=None, nuc=None):
    """uint16 volume (z, y, x) of slices [z_begin, z_end)."""
    z_end = s.depth if z_end is None else z_end
    if nuc is None:
        nuc = nuclei(s)
    nuc = np.ascontiguousarray(nuc, np.float64)
    out = np.empty((z_end - z_begin, s.height, s.width), np.uint16)
    rc = _L().hdog_synth_render(ctypes.byref(s), nuc.ctypes.data, nuc.shape[0], z_begin, z_end, out.ctypes.data)
    if rc != 0:
        raise HDoGError(HDOG_ERR_ARG, "render failed")
    return out


def clustered_nuclei(w, h, d, total, seed, cluster_fraction=0.3, sizes=(2, 6)):
    """`total` nuclei, `cluster_fraction` of them in clusters of sizes[0]..sizes[1] members
    (the dense streaming stack): a cluster's extra members touch its first one, at centre
    distance 0.8 (sigma_a + sigma_b) along a random direction (the z offset scaled by
    sigma_z / sigma_xy).  Rows as nuclei(): x, y, z, sigma_xy, sigma_z, peak."""
    rng = np.random.default_rng(seed)
    n_cl = int(cluster_fraction * total)
    cs = rng.integers(sizes[0], sizes[1] + 1, size=n_cl // sizes[0] + 1)
    cs = cs[: np.searchsorted(np.cumsum(cs), n_cl) + 1]
    n_seed = total - int(cs.sum()) + len(cs)
    base = nuclei(spec(w, h, d, n_seed, seed))
    first = np.repeat(np.arange(len(cs)), cs - 1)            # the cluster each extra member joins
    extra = base[rng.integers(len(base), size=len(first))].copy()
    v = rng.normal(size=(len(first), 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    a = base[first]
    dist = 0.8 * (a[:, 3] + extra[:, 3])
    extra[:, :3] = a[:, :3] + v * np.stack([dist, dist, dist * a[:, 4] / a[:, 3]], axis=1)
    keep = (extra[:, 0] >= 0) & (extra[:, 0] < w) & (extra[:, 1] >= 0) & (extra[:, 1] < h) & \
           (extra[:, 2] >= 0) & (extra[:, 2] < d)
    return np.concatenate([base, extra[keep]])
