"""The differentiable HDoG chain as a torch.autograd.Function over libhdog's hand-written
forward and adjoint kernels (hdog_soft_forward / hdog_soft_backward): normalize -> DoG ->
Hessian -> the mask test relaxed to a product of sigmoids, scored at positive and negative
sample points.  Torch only holds the tensors and the graph; every stage runs in libhdog.

    loss = hdog.soft.soft_loss(volume, sigma, pos, neg, radius_norm_xy=20, radius_norm_z=5,
                               min_intensity=50.0, tau=1e-3)
    loss.backward()      # volume.grad, sigma.grad

volume: (D, H, W) float32 CUDA tensor; sigma: 6 values (x1, y1, z1, x2, y2, z2; the small
then the large scale); pos / neg: (n, 3) int32 CUDA tensors of (z, y, x) voxel indices.
"""
import ctypes

import torch

from . import check, hdog_soft_params, lib


def _params(vol, sigma, cfg):
    rxy, rz, min_intensity, tau, gamma = cfg
    D, H, W = vol.shape
    s = [float(v) for v in sigma.detach().cpu().reshape(-1)]
    assert len(s) == 6, "sigma holds 6 values: x1, y1, z1, x2, y2, z2"
    return hdog_soft_params(int(W), int(H), int(D), int(rxy), int(rz), float(min_intensity), (ctypes.c_float * 6)(*s),
                            float(gamma), float(tau))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else None


def _check_inputs(vol, pos, neg):
    assert vol.is_cuda and vol.dtype == torch.float32 and vol.dim() == 3 and vol.is_contiguous()
    for p in (pos, neg):
        assert p.is_cuda and p.dtype == torch.int32 and p.dim() == 2 and p.shape[1] == 3 and p.is_contiguous()


class SoftLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vol, sigma, pos, neg, cfg):
        _check_inputs(vol, pos, neg)
        p = _params(vol, sigma, cfg)
        ws = torch.empty(lib().hdog_soft_workspace_bytes(ctypes.byref(p)), dtype=torch.uint8, device=vol.device)
        loss = torch.empty(1, dtype=torch.float32, device=vol.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(vol.device).cuda_stream)
        check(lib().hdog_soft_forward(ctypes.byref(p), _ptr(vol), _ptr(pos), pos.shape[0], _ptr(neg), neg.shape[0],
                                      _ptr(loss), None, _ptr(ws), stream))
        ctx.save_for_backward(vol, sigma, pos, neg)
        ctx.cfg = cfg
        return loss[0]

    @staticmethod
    def backward(ctx, grad):
        vol, sigma, pos, neg = ctx.saved_tensors
        p = _params(vol, sigma, ctx.cfg)
        want_vol, want_sigma = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        gv = torch.zeros_like(vol) if want_vol else None
        gs = torch.zeros(6, dtype=torch.float32, device=vol.device) if want_sigma else None
        ws = torch.empty(lib().hdog_soft_workspace_bytes(ctypes.byref(p)), dtype=torch.uint8, device=vol.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(vol.device).cuda_stream)
        check(lib().hdog_soft_backward(ctypes.byref(p), _ptr(vol), _ptr(pos), pos.shape[0], _ptr(neg), neg.shape[0],
                                       float(grad), _ptr(gv), _ptr(gs), _ptr(ws), stream))
        if gs is not None:
            gs = gs.to(device=sigma.device, dtype=sigma.dtype).reshape(sigma.shape)
        return gv, gs, None, None, None


def soft_loss(vol, sigma, pos, neg, radius_norm_xy=20, radius_norm_z=5, min_intensity=50.0, tau=1e-3, gamma=1.0):
    """Mean relaxed mask score at pos minus that at neg (see the module docstring)."""
    return SoftLoss.apply(vol, sigma, pos, neg, (radius_norm_xy, radius_norm_z, min_intensity, tau, gamma))


def fit_sigmas(vol, pos, neg, sigma0, steps=20, lr=0.05, **kw):
    """Gradient ascent on the loss over the six DoG sigmas (Adam), the tap radii re-derived
    from the sigmas at every step; returns (sigmas, loss history)."""
    sigma = torch.tensor([float(v) for v in sigma0], dtype=torch.float32, requires_grad=True)
    opt = torch.optim.Adam([sigma], lr=lr)
    history = []
    for _ in range(steps):
        opt.zero_grad()
        loss = soft_loss(vol, sigma, pos, neg, **kw)
        (-loss).backward()
        opt.step()
        with torch.no_grad():
            sigma.clamp_(min=0.3)
        history.append(float(loss.detach()))
    return sigma.detach(), history
