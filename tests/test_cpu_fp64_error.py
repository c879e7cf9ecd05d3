"""The float volumes' error against FP64, stated.  The CUDA path equals the FP32 oracle bit
for bit (the stage tests), so the oracle's error is this library's.  The FP64 references
compute the same operators in float64: min / max exactly, box means over the nearest border,
the reference's Gaussian taps (the float coefficients themselves, as float64) with zero
borders, and the Hessian's central differences with zero halos.  Errors are relative to the
largest magnitude of each volume, over the voxels where the normalization is finite."""
import numpy as np
import torch

from helpers import volume
from oracle import oracle as orc
from oracle import soft_ref as sr

RXY, RZ, MIN_I = 20, 5, 50.0
SIG = (2.0, 1.5, 3.2, 2.4)


def conv_f64(x, taps, axis):
    r = (len(taps) - 1) // 2
    xp = np.pad(x, [(r, r) if a == axis else (0, 0) for a in range(3)])
    out = np.zeros_like(x)
    n = x.shape[axis]
    for j in range(-r, r + 1):
        out += taps[r - j] * np.take(xp, np.arange(n) + r + j, axis=axis)
    return out


def gauss_f64(x, sxy, sz):
    kxy, rxy = orc.gauss_taps(sxy)
    kz, rz = orc.gauss_taps(sz)
    kxy = kxy[:2 * rxy + 1].astype(np.float64)
    kz = kz[:2 * rz + 1].astype(np.float64)
    return conv_f64(conv_f64(conv_f64(x, kxy, 2), kxy, 1), kz, 0)


def test_float_volumes_against_fp64():
    vol = volume(96, 96, 40, n_nuclei=60, seed=99)
    n32 = orc.normalize(vol, RXY, RZ, MIN_I)
    n64 = sr.normalize(torch.tensor(vol, dtype=torch.float64), RXY, RZ, MIN_I).numpy()
    ok = np.isfinite(n64) & np.isfinite(n32)
    assert ok.mean() > 0.99
    e_norm = np.abs(n32[ok] - n64[ok]).max() / np.abs(n64[ok]).max()
    nz = np.where(ok, n64, 0.0)
    nrm = float(orc.dog_normalizer(SIG[0], SIG[1], 1.0))
    d64 = (gauss_f64(nz, SIG[0], SIG[1]) - gauss_f64(nz, SIG[2], SIG[3])) * nrm
    d32 = orc.dog(np.where(ok, n32, 0.0).astype(np.float32), *SIG, 1.0)
    e_dog = np.abs(d32 - d64).max() / np.abs(d64).max()
    _, h32 = orc.hessian_pd(d32, want_hessian=True)
    h64 = sr.hessian(torch.tensor(d64))
    e_h = max(np.abs(h32[k] - h64[k].numpy()).max() / np.abs(h64[k].numpy()).max() for k in range(6))
    print("max error / max magnitude vs FP64: normalized %.2e, DoG %.2e, Hessian elements %.2e"
          % (e_norm, e_dog, e_h))
    assert e_norm < 1e-6 and e_dog < 1e-5 and e_h < 1e-4
