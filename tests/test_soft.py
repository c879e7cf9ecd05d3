"""The differentiable chain (normalize -> DoG -> Hessian -> relaxed mask score): the FP64
torch reference (oracle/soft_ref.py) against FP64 central differences on CPU, and libhdog's
float32 forward / hand-written adjoint against that reference on the GPU.

Tolerances: loss within 1e-5 relative of the FP64 reference; sigma gradients within 1e-4
relative of the FP64 reference gradient and of FP64 central differences (step 1e-3);
input gradients within 1e-4 of the largest input-gradient magnitude, elementwise.  The
test volume carries a fractional part on every voxel, so no min / max window has a tie
(at a tie the filters are not differentiable and central differences average the sides).
"""
import numpy as np
import pytest
import torch

from oracle import soft_ref as sr

D, H, W = 14, 40, 44
RXY, RZ, MIN_INT = 4, 2, 50.0
SIGMA = [1.2, 1.3, 1.1, 1.9, 2.1, 1.7]
BLOBS = [(6, 12, 14), (7, 26, 30), (5, 30, 10), (8, 14, 33)]


def case():
    rng = np.random.default_rng(20261203)
    vol = 100 + rng.normal(0, 8, (D, H, W)) + rng.uniform(0, 1, (D, H, W))
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    for c in BLOBS:
        vol += 800 * np.exp(-((xx - c[2]) ** 2 / (2 * 2.2 ** 2) + (yy - c[1]) ** 2 / (2 * 2.2 ** 2) +
                              (zz - c[0]) ** 2 / (2 * 1.5 ** 2)))
    pos = np.array([[z + dz, y + dy, x] for (z, y, x) in BLOBS for dz, dy in ((0, 0), (1, 0), (0, 1))], np.int32)
    neg = np.stack([rng.integers(0, D, 12), rng.integers(0, H, 12), rng.integers(0, W, 12)], 1).astype(np.int32)
    return vol, pos, neg


def ref_tau(vol, pos):
    with torch.no_grad():
        h = sr.hessian(sr.dog(sr.normalize(torch.tensor(vol), RXY, RZ, MIN_INT),
                              [torch.tensor(v, dtype=torch.float64) for v in SIGMA]))
        return float(torch.stack([e[pos[:, 0], pos[:, 1], pos[:, 2]].abs() for e in h]).median())


def ref_loss_and_grads(vol, pos, neg, tau):
    I = torch.tensor(vol, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(SIGMA, dtype=torch.float64, requires_grad=True)
    L = sr.loss(I, list(sig), torch.tensor(pos, dtype=torch.long), torch.tensor(neg, dtype=torch.long), RXY, RZ,
                MIN_INT, tau)
    L.backward()
    return float(L.detach()), I.grad.numpy(), sig.grad.numpy()


def ref_loss(vol, sig, pos, neg, tau):
    with torch.no_grad():
        return float(sr.loss(torch.tensor(vol), [torch.tensor(v, dtype=torch.float64) for v in sig],
                             torch.tensor(pos, dtype=torch.long), torch.tensor(neg, dtype=torch.long),
                             RXY, RZ, MIN_INT, tau))


@pytest.fixture(scope="module")
def reference():
    vol, pos, neg = case()
    tau = ref_tau(vol, pos)
    L, gI, gs = ref_loss_and_grads(vol, pos, neg, tau)
    return vol, pos, neg, tau, L, gI, gs


def test_reference_gradient_matches_central_differences(reference):
    vol, pos, neg, tau, L, gI, gs = reference
    h = 1e-3
    for k in range(6):
        sp, sm = list(SIGMA), list(SIGMA)
        sp[k] += h
        sm[k] -= h
        fd = (ref_loss(vol, sp, pos, neg, tau) - ref_loss(vol, sm, pos, neg, tau)) / (2 * h)
        assert abs(fd - gs[k]) <= 1e-4 * max(abs(gs[k]), 1e-12) + 1e-10, (k, fd, gs[k])
    for v in list(zip(*np.unravel_index(np.argsort(-np.abs(gI).ravel())[:6], gI.shape))):
        vp, vm = vol.copy(), vol.copy()
        vp[v] += h
        vm[v] -= h
        fd = (ref_loss(vp, SIGMA, pos, neg, tau) - ref_loss(vm, SIGMA, pos, neg, tau)) / (2 * h)
        assert abs(fd - gI[v]) <= 1e-4 * abs(gI[v]) + 1e-12, (v, fd, gI[v])


@pytest.mark.gpu
def test_gpu_forward_and_adjoint_match_reference(reference):
    import hdog
    vol, pos, neg, tau, L, gI, gs = reference
    v = torch.tensor(vol, dtype=torch.float32, device="cuda", requires_grad=True)
    s = torch.tensor(SIGMA, dtype=torch.float32, requires_grad=True)
    loss = hdog.soft.soft_loss(v, s, torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda"),
                               radius_norm_xy=RXY, radius_norm_z=RZ, min_intensity=MIN_INT, tau=tau)
    loss.backward()
    lv = float(loss.detach())
    assert abs(lv - L) <= 1e-5 * abs(L), (lv, L)
    g_s = s.grad.numpy().astype(np.float64)
    assert np.all(np.abs(g_s - gs) <= 1e-4 * np.abs(gs) + 1e-9), (g_s, gs)
    g_v = v.grad.cpu().numpy().astype(np.float64)
    scale = np.abs(gI).max()
    err = np.abs(g_v - gI)
    assert err.max() <= 1e-4 * scale, (float(err.max()), scale)


@pytest.mark.gpu
def test_gpu_sigma_fit_improves_the_loss(reference):
    import hdog
    vol, pos, neg, tau, L, gI, gs = reference
    v = torch.tensor(vol, dtype=torch.float32, device="cuda")
    start = [1.6, 1.6, 1.6, 2.6, 2.6, 2.6]
    sig, hist = hdog.soft.fit_sigmas(v, torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda"), start,
                                     steps=15, lr=0.05, radius_norm_xy=RXY, radius_norm_z=RZ, min_intensity=MIN_INT,
                                     tau=tau)
    assert hist[-1] > hist[0] + 1e-3, hist
