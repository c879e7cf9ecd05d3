"""The differentiable HDoG chain as a torch.autograd.Function over libhdog's hand-written
forward and adjoint kernels (hdog_soft_forward / hdog_soft_backward): normalize -> DoG ->
Hessian -> the mask test relaxed to a product of sigmoids, scored at positive and negative
sample points.  Torch only holds the tensors and the graph; every stage runs in libhdog.

    loss = hdog.soft.soft_loss(volume, sigma, pos, neg, thresh=b, radius_norm_xy=20,
                               radius_norm_z=5, min_intensity=50.0, tau=1e-3)
    loss.backward()      # volume.grad, sigma.grad, b.grad

By default the forward's workspace (17 volume-sized float32 buffers) stays alive until the
backward, which then takes the forward chain's intermediates from it instead of recomputing
them (same results); keep_intermediates=False frees it after the forward and the backward
recomputes.

volume: (D, H, W) float32 CUDA tensor; sigma: 6 values (x1, y1, z1, x2, y2, z2; the small
then the large scale); thresh: 3 offsets (b0, b1, b2) of the relaxed tests xx < b0,
xx yy - xy^2 > b1, det < b2 (zero: the reference's mask test), optional; pos / neg: (n, 3)
int32 CUDA tensors of (z, y, x) voxel indices.
"""
import ctypes

import torch

from . import check, hdog_soft_params, lib


def _params(vol, sigma, thresh, cfg):
    rxy, rz, min_intensity, tau, gamma = cfg
    D, H, W = vol.shape
    s = [float(v) for v in sigma.detach().cpu().reshape(-1)]
    assert len(s) == 6, "sigma holds 6 values: x1, y1, z1, x2, y2, z2"
    b = [float(v) for v in thresh.detach().cpu().reshape(-1)]
    assert len(b) == 3, "thresh holds 3 values: b0, b1, b2"
    return hdog_soft_params(int(W), int(H), int(D), int(rxy), int(rz), float(min_intensity), (ctypes.c_float * 6)(*s),
                            float(gamma), float(tau), (ctypes.c_float * 3)(*b))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else None


def _check_inputs(vol, pos, neg):
    assert vol.is_cuda and vol.dtype == torch.float32 and vol.dim() == 3 and vol.is_contiguous()
    for p in (pos, neg):
        assert p.is_cuda and p.dtype == torch.int32 and p.dim() == 2 and p.shape[1] == 3 and p.is_contiguous()


class SoftLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vol, sigma, thresh, pos, neg, cfg, keep):
        _check_inputs(vol, pos, neg)
        p = _params(vol, sigma, thresh, cfg)
        ws = torch.empty(lib().hdog_soft_workspace_bytes(ctypes.byref(p)), dtype=torch.uint8, device=vol.device)
        loss = torch.empty(1, dtype=torch.float32, device=vol.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(vol.device).cuda_stream)
        check(lib().hdog_soft_forward(ctypes.byref(p), _ptr(vol), _ptr(pos), pos.shape[0], _ptr(neg), neg.shape[0],
                                      _ptr(loss), None, _ptr(ws), stream))
        ctx.save_for_backward(vol, sigma, thresh, pos, neg)
        ctx.cfg = cfg
        # the saved tensors' version check already refuses a volume changed in place since
        ctx.kept = ws if keep else None
        return loss[0]

    @staticmethod
    def backward(ctx, grad):
        vol, sigma, thresh, pos, neg = ctx.saved_tensors
        p = _params(vol, sigma, thresh, ctx.cfg)
        want_vol, want_sigma, want_thresh = ctx.needs_input_grad[0], ctx.needs_input_grad[1], ctx.needs_input_grad[2]
        gv = torch.zeros_like(vol) if want_vol else None
        gs = torch.zeros(6, dtype=torch.float32, device=vol.device) if want_sigma else None
        gb = torch.zeros(3, dtype=torch.float32, device=vol.device) if want_thresh else None
        stream = ctypes.c_void_p(torch.cuda.current_stream(vol.device).cuda_stream)
        if ctx.kept is not None:
            ws = ctx.kept
            fn = lib().hdog_soft_backward_kept
        else:
            ws = torch.empty(lib().hdog_soft_workspace_bytes(ctypes.byref(p)), dtype=torch.uint8, device=vol.device)
            fn = lib().hdog_soft_backward
        check(fn(ctypes.byref(p), _ptr(vol), _ptr(pos), pos.shape[0], _ptr(neg), neg.shape[0], float(grad), _ptr(gv),
                 _ptr(gs), _ptr(gb), _ptr(ws), stream))
        if gs is not None:
            gs = gs.to(device=sigma.device, dtype=sigma.dtype).reshape(sigma.shape)
        if gb is not None:
            gb = gb.to(device=thresh.device, dtype=thresh.dtype).reshape(thresh.shape)
        return gv, gs, gb, None, None, None, None


def soft_loss(vol, sigma, pos, neg, thresh=None, radius_norm_xy=20, radius_norm_z=5, min_intensity=50.0, tau=1e-3,
              gamma=1.0, keep_intermediates=True):
    """Mean relaxed mask score at pos minus that at neg (see the module docstring)."""
    if thresh is None:
        thresh = torch.zeros(3, dtype=torch.float32)
    pos, neg = pos.contiguous(), neg.contiguous()
    return SoftLoss.apply(vol, sigma, thresh, pos, neg, (radius_norm_xy, radius_norm_z, min_intensity, tau, gamma),
                          bool(keep_intermediates))


def fit(vol, pos, neg, sigma0, thresh0=(0.0, 0.0, 0.0), steps=20, lr=0.05, lr_thresh=None, fit_thresholds=True,
        **kw):
    """Gradient ascent on the loss (Adam) over the six DoG sigmas and, unless fit_thresholds
    is False, the three test thresholds -- the sweep of sigmas and thresholds the reference
    leaves to the user, done by gradient; tap radii are re-derived from the sigmas at every
    step.  lr_thresh defaults to lr times tau (the thresholds live on the scale of the
    Hessian elements).  Returns (sigmas, thresholds, loss history)."""
    sigma = torch.tensor([float(v) for v in sigma0], dtype=torch.float32, requires_grad=True)
    thresh = torch.tensor([float(v) for v in thresh0], dtype=torch.float32, requires_grad=fit_thresholds)
    groups = [{"params": [sigma], "lr": lr}]
    if fit_thresholds:
        tau = kw.get("tau", 1e-3)
        groups.append({"params": [thresh], "lr": lr * tau if lr_thresh is None else lr_thresh})
    opt = torch.optim.Adam(groups)
    history = []
    for _ in range(steps):
        opt.zero_grad()
        loss = soft_loss(vol, sigma, pos, neg, thresh=thresh, **kw)
        (-loss).backward()
        opt.step()
        with torch.no_grad():
            sigma.clamp_(min=0.3)
        history.append(float(loss.detach()))
    return sigma.detach(), thresh.detach(), history


def fit_sigmas(vol, pos, neg, sigma0, steps=20, lr=0.05, **kw):
    """fit() over the six DoG sigmas alone, the thresholds held at zero; returns (sigmas, loss
    history)."""
    sigma, _, history = fit(vol, pos, neg, sigma0, steps=steps, lr=lr, fit_thresholds=False, **kw)
    return sigma, history
