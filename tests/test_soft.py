"""The differentiable chain (normalize -> DoG -> Hessian -> relaxed mask score): the FP64
torch reference (oracle/soft_ref.py) against FP64 central differences on CPU, and libhdog's
float32 forward / hand-written adjoint against that reference on the GPU.

Tolerances: loss within 1e-5 relative of the FP64 reference; sigma and threshold
gradients within 1e-4 relative of the FP64 reference gradient and of FP64 central
differences (step 1e-3, thresholds stepped by 1e-3 of their scale tau^k); input gradients
within 1e-4 of the largest input-gradient magnitude, elementwise.  The test volume carries a
fractional part on every voxel, so no min / max window has a tie (at a tie the filters are
not differentiable and central differences average the sides).  The thresholds are set off
zero, so their gradients are not a symmetric special case.
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


def thresholds(tau):
    """Test thresholds off zero, on each test's scale."""
    return [0.15 * tau, -0.2 * tau ** 2, 0.1 * tau ** 3]


def ref_loss_and_grads(vol, pos, neg, tau, b):
    I = torch.tensor(vol, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(SIGMA, dtype=torch.float64, requires_grad=True)
    bt = torch.tensor(b, dtype=torch.float64, requires_grad=True)
    L = sr.loss(I, list(sig), torch.tensor(pos, dtype=torch.long), torch.tensor(neg, dtype=torch.long), RXY, RZ,
                MIN_INT, tau, b=list(bt))
    L.backward()
    return float(L.detach()), I.grad.numpy(), sig.grad.numpy(), bt.grad.numpy()


def ref_loss(vol, sig, pos, neg, tau, b):
    with torch.no_grad():
        return float(sr.loss(torch.tensor(vol), [torch.tensor(v, dtype=torch.float64) for v in sig],
                             torch.tensor(pos, dtype=torch.long), torch.tensor(neg, dtype=torch.long),
                             RXY, RZ, MIN_INT, tau, b=[torch.tensor(v, dtype=torch.float64) for v in b]))


@pytest.fixture(scope="module")
def reference():
    vol, pos, neg = case()
    tau = ref_tau(vol, pos)
    b = thresholds(tau)
    L, gI, gs, gb = ref_loss_and_grads(vol, pos, neg, tau, b)
    return vol, pos, neg, tau, b, L, gI, gs, gb


def test_reference_gradient_matches_central_differences(reference):
    vol, pos, neg, tau, b, L, gI, gs, gb = reference
    h = 1e-3
    for k in range(6):
        sp, sm = list(SIGMA), list(SIGMA)
        sp[k] += h
        sm[k] -= h
        fd = (ref_loss(vol, sp, pos, neg, tau, b) - ref_loss(vol, sm, pos, neg, tau, b)) / (2 * h)
        assert abs(fd - gs[k]) <= 1e-4 * max(abs(gs[k]), 1e-12) + 1e-10, (k, fd, gs[k])
    for k in range(3):
        hk = h * tau ** (k + 1)
        bp, bm = list(b), list(b)
        bp[k] += hk
        bm[k] -= hk
        fd = (ref_loss(vol, SIGMA, pos, neg, tau, bp) - ref_loss(vol, SIGMA, pos, neg, tau, bm)) / (2 * hk)
        assert abs(fd - gb[k]) <= 1e-4 * abs(gb[k]), (k, fd, gb[k])
    for v in list(zip(*np.unravel_index(np.argsort(-np.abs(gI).ravel())[:6], gI.shape))):
        vp, vm = vol.copy(), vol.copy()
        vp[v] += h
        vm[v] -= h
        fd = (ref_loss(vp, SIGMA, pos, neg, tau, b) - ref_loss(vm, SIGMA, pos, neg, tau, b)) / (2 * h)
        assert abs(fd - gI[v]) <= 1e-4 * abs(gI[v]) + 1e-12, (v, fd, gI[v])


@pytest.mark.gpu
def test_gpu_forward_and_adjoint_match_reference(reference):
    import hdog
    vol, pos, neg, tau, b, L, gI, gs, gb = reference
    v = torch.tensor(vol, dtype=torch.float32, device="cuda", requires_grad=True)
    s = torch.tensor(SIGMA, dtype=torch.float32, requires_grad=True)
    bt = torch.tensor(b, dtype=torch.float32, requires_grad=True)
    loss = hdog.soft.soft_loss(v, s, torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda"), thresh=bt,
                               radius_norm_xy=RXY, radius_norm_z=RZ, min_intensity=MIN_INT, tau=tau)
    loss.backward()
    lv = float(loss.detach())
    assert abs(lv - L) <= 1e-5 * abs(L), (lv, L)
    g_s = s.grad.numpy().astype(np.float64)
    assert np.all(np.abs(g_s - gs) <= 1e-4 * np.abs(gs) + 1e-9), (g_s, gs)
    g_b = bt.grad.numpy().astype(np.float64)
    assert np.all(np.abs(g_b - gb) <= 1e-4 * np.abs(gb)), (g_b, gb)
    g_v = v.grad.cpu().numpy().astype(np.float64)
    scale = np.abs(gI).max()
    err = np.abs(g_v - gI)
    assert err.max() <= 1e-4 * scale, (float(err.max()), scale)


@pytest.mark.gpu
@pytest.mark.parametrize("rxy,rz", [(20, 5), (40, 3)])
def test_gpu_adjoint_with_wide_normalization_windows(rxy, rz):
    """The case above with the workload's normalization reach (20, 5) and with a reach of 40
    (wider than the lines; the x tiles up to 64, the y / z min / max kernels up to 32, the
    y / z tiles above), against the FP64 reference gradient.  The sigma gradients are held to
    2e-4 relative here: the float32 box means sum 41 values per axis, and the sigma gradients,
    which go through second differences of the DoG and sigmoids scaled by 1/tau^3, move by
    about 1e-4 for a last-bit change of the normalized volume (measured: 1.22e-4 on sigma_y1
    at reach 20; min / max do not round, so this is the float32 rounding of the box means and
    Gaussians); the loss, threshold and input gradients keep the bounds above."""
    import hdog
    vol, pos, neg = case()
    with torch.no_grad():
        h = sr.hessian(sr.dog(sr.normalize(torch.tensor(vol), rxy, rz, MIN_INT),
                              [torch.tensor(v, dtype=torch.float64) for v in SIGMA]))
        tau = float(torch.stack([e[pos[:, 0], pos[:, 1], pos[:, 2]].abs() for e in h]).median())
    b = thresholds(tau)
    I = torch.tensor(vol, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(SIGMA, dtype=torch.float64, requires_grad=True)
    bt = torch.tensor(b, dtype=torch.float64, requires_grad=True)
    L = sr.loss(I, list(sig), torch.tensor(pos, dtype=torch.long), torch.tensor(neg, dtype=torch.long), rxy, rz,
                MIN_INT, tau, b=list(bt))
    L.backward()
    v = torch.tensor(vol, dtype=torch.float32, device="cuda", requires_grad=True)
    s = torch.tensor(SIGMA, dtype=torch.float32, requires_grad=True)
    b32 = torch.tensor(b, dtype=torch.float32, requires_grad=True)
    loss = hdog.soft.soft_loss(v, s, torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda"), thresh=b32,
                               radius_norm_xy=rxy, radius_norm_z=rz, min_intensity=MIN_INT, tau=tau)
    loss.backward()
    assert abs(float(loss.detach()) - float(L.detach())) <= 1e-5 * abs(float(L.detach()))
    gs = sig.grad.numpy()
    assert np.all(np.abs(s.grad.numpy() - gs) <= 2e-4 * np.abs(gs) + 1e-9), (s.grad.numpy(), gs)
    gb = bt.grad.numpy()
    assert np.all(np.abs(b32.grad.numpy() - gb) <= 1e-4 * np.abs(gb)), (b32.grad.numpy(), gb)
    gI = I.grad.numpy()
    err = np.abs(v.grad.cpu().numpy().astype(np.float64) - gI)
    assert err.max() <= 1e-4 * np.abs(gI).max(), (float(err.max()), float(np.abs(gI).max()))


@pytest.mark.gpu
def test_gpu_backward_from_the_kept_forward_equals_the_recomputed_one(reference):
    """The backward that takes the forward's intermediates from its workspace (the default)
    against the one that recomputes them, and two backward calls after one forward: the
    same gradients up to the order of the double and float atomic sums (a last-bit effect)."""
    import hdog
    vol, pos, neg, tau, b = reference[:5]
    p, n = torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda")

    def grads(keep, calls=1):
        v = torch.tensor(vol, dtype=torch.float32, device="cuda", requires_grad=True)
        s = torch.tensor(SIGMA, dtype=torch.float32, requires_grad=True)
        bt = torch.tensor(b, dtype=torch.float32, requires_grad=True)
        loss = hdog.soft.soft_loss(v, s, p, n, thresh=bt, radius_norm_xy=RXY, radius_norm_z=RZ,
                                   min_intensity=MIN_INT, tau=tau, keep_intermediates=keep)
        for k in range(calls):
            loss.backward(retain_graph=k + 1 < calls)
        return v.grad.cpu().numpy() / calls, s.grad.numpy() / calls, bt.grad.numpy() / calls

    kept, again, recomputed = grads(True), grads(True, calls=2), grads(False)
    for g in (again, recomputed):
        for a, r in zip(kept, g):
            assert np.allclose(a, r, rtol=1e-6, atol=1e-6 * np.abs(r).max()), (np.abs(a - r).max(), np.abs(r).max())


@pytest.mark.gpu
def test_gpu_sigma_fit_improves_the_loss(reference):
    import hdog
    vol, pos, neg, tau = reference[:4]
    v = torch.tensor(vol, dtype=torch.float32, device="cuda")
    start = [1.6, 1.6, 1.6, 2.6, 2.6, 2.6]
    sig, hist = hdog.soft.fit_sigmas(v, torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda"), start,
                                     steps=15, lr=0.05, radius_norm_xy=RXY, radius_norm_z=RZ, min_intensity=MIN_INT,
                                     tau=tau)
    assert hist[-1] > hist[0] + 1e-3, hist


@pytest.mark.gpu
def test_gpu_fit_of_sigmas_and_thresholds_beats_sigmas_alone(reference):
    import hdog
    vol, pos, neg, tau = reference[:4]
    v = torch.tensor(vol, dtype=torch.float32, device="cuda")
    p, n = torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda")
    start = [1.6, 1.6, 1.6, 2.6, 2.6, 2.6]
    kw = dict(steps=15, lr=0.05, radius_norm_xy=RXY, radius_norm_z=RZ, min_intensity=MIN_INT, tau=tau)
    _, hs = hdog.soft.fit_sigmas(v, p, n, start, **kw)
    sig, b, hb = hdog.soft.fit(v, p, n, start, **kw)
    assert hb[-1] > hb[0] + 1e-3, hb
    assert hb[-1] >= hs[-1] - 1e-4, (hb[-1], hs[-1])
    assert np.any(b.numpy() != 0.0)


CROP = (24, 72, 80)   # (D, H, W) crop of a 128 x 512 x 512 volume of the differentiable workload


@pytest.mark.gpu
def test_gpu_adjoint_on_a_crop_of_the_workload_volume():
    """The adjoint on a crop of a seeded 128 x 512 x 512 synthetic volume (3200 nuclei, the
    differentiable workload's generator), with sample points at nucleus centroids and random
    voxels inside the crop, against the FP64 reference gradient."""
    import hdog
    from hdog import synth
    spec = synth.spec(512, 512, 128, 3200, synth.SEED_BASE + 300)
    nuc = synth.nuclei(spec)
    z0, y0, x0 = 52, 200, 216
    D_, H_, W_ = CROP
    vol = synth.volume(spec, z0, z0 + D_, nuc=nuc)[:, y0:y0 + H_, x0:x0 + W_].astype(np.float64)
    vol += np.random.default_rng(7).uniform(0, 1, vol.shape)     # no ties in the min / max windows
    inside = nuc[(nuc[:, 0] >= x0 + 4) & (nuc[:, 0] < x0 + W_ - 4) & (nuc[:, 1] >= y0 + 4) &
                 (nuc[:, 1] < y0 + H_ - 4) & (nuc[:, 2] >= z0 + 3) & (nuc[:, 2] < z0 + D_ - 3)]
    assert len(inside) >= 3
    pos = np.ascontiguousarray(np.rint(inside[:, [2, 1, 0]] - [z0, y0, x0]).astype(np.int32))
    rng = np.random.default_rng(8)
    neg = np.stack([rng.integers(0, D_, 40), rng.integers(0, H_, 40), rng.integers(0, W_, 40)], 1).astype(np.int32)
    rxy, rz = 6, 3
    with torch.no_grad():
        h = sr.hessian(sr.dog(sr.normalize(torch.tensor(vol), rxy, rz, 50.0),
                              [torch.tensor(x, dtype=torch.float64) for x in SIGMA]))
        tau = float(torch.stack([e[pos[:, 0], pos[:, 1], pos[:, 2]].abs() for e in h]).median())
    b = thresholds(tau)
    I = torch.tensor(vol, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(SIGMA, dtype=torch.float64, requires_grad=True)
    bt = torch.tensor(b, dtype=torch.float64, requires_grad=True)
    L = sr.loss(I, list(sig), torch.tensor(pos, dtype=torch.long), torch.tensor(neg, dtype=torch.long), rxy, rz,
                50.0, tau, b=list(bt))
    L.backward()
    v = torch.tensor(vol, dtype=torch.float32, device="cuda", requires_grad=True)
    s = torch.tensor(SIGMA, dtype=torch.float32, requires_grad=True)
    b32 = torch.tensor(b, dtype=torch.float32, requires_grad=True)
    loss = hdog.soft.soft_loss(v, s, torch.tensor(pos, device="cuda"), torch.tensor(neg, device="cuda"), thresh=b32,
                               radius_norm_xy=rxy, radius_norm_z=rz, min_intensity=50.0, tau=tau)
    loss.backward()
    assert abs(float(loss.detach()) - float(L.detach())) <= 1e-5 * abs(float(L.detach()))
    gs = sig.grad.numpy()
    assert np.all(np.abs(s.grad.numpy() - gs) <= 1e-4 * np.abs(gs) + 1e-9), (s.grad.numpy(), gs)
    gb = bt.grad.numpy()
    assert np.all(np.abs(b32.grad.numpy() - gb) <= 1e-4 * np.abs(gb)), (b32.grad.numpy(), gb)
    gI = I.grad.numpy()
    err = np.abs(v.grad.cpu().numpy().astype(np.float64) - gI)
    assert err.max() <= 1e-4 * np.abs(gI).max(), (float(err.max()), float(np.abs(gI).max()))
