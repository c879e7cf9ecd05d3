"""TEST INFRASTRUCTURE (the oracle): FP64 reference of the differentiable HDoG chain, in
torch float64 on the CPU with autograd.  Only tests/ (and bench.py's differentiable
workload, as its checker) use it; the product path is libhdog's adjoint kernels.

The chain follows the reference's forward stages with their borders (and the
differentiable relaxation of its mask):
  normalize   NormalizeFilter.cu:537-654: min / max over a (2r_xy+1)^2 (2r_z+1) box with
              nearest borders, their box means (nearest borders), norm = I >= min_intensity ?
              (I - ero) / (dil - ero) : 0
  DoG         DoG3DFilter.cu:70-437: separable Gaussians with zero borders, taps
              exp(-k^2 / 2 sigma^2) normalized to sum 1 over |k| <= (int)(2 sigma + 0.5),
              dog = (G_small - G_large) norm * normalizer; here each axis has its own sigma
              (sigma_x, sigma_y, sigma_z per scale) and normalizer = (sx1 sy1 sz1)^gamma, which is
              the reference's sxy1^(2 gamma) sz1^gamma when sx1 = sy1
  Hessian     Hessian3DFilter_element.cu:22-388: central differences of central differences,
              values outside the volume 0 and first derivatives at positions outside the
              volume 0; element order xx, xy, xz, yy, yz, zz
  soft score  the leading-principal-minor test xx < 0, xx yy - xy^2 > 0, det < 0
              (PositiveDefiniteKernel, Hessian3DFilter_element.cu:317-321) with thresholds
              b relaxed to sigmoid((b0 - xx) / tau) * sigmoid((xx yy - xy^2 - b1) / tau^2) *
              sigmoid((b2 - det) / tau^3)
  loss        mean score at the positive points minus mean score at the negative points
The tap radius is a step function of sigma and is held fixed for derivatives.
"""
import torch
import torch.nn.functional as F


def taps(sigma):
    """Normalized Gaussian taps for sigma (a float64 scalar tensor), radius int(2 sigma + 0.5)."""
    r = int(2.0 * float(sigma.detach()) + 0.5)
    k = torch.arange(-r, r + 1, dtype=torch.float64)
    t = torch.exp(-0.5 * k * k / (sigma * sigma))
    return t / t.sum()


def _along(x, axis, fn):
    """Applies fn over the last dimension with `axis` (0 z, 1 y, 2 x of a (D, H, W) volume) moved there."""
    x = x.movedim(axis, -1)
    shape = x.shape
    y = fn(x.reshape(-1, 1, shape[-1]))
    return y.reshape(shape[:-1] + (y.shape[-1],)).movedim(-1, axis)


def minmax1d(x, axis, r, is_max):
    if r == 0:
        return x
    def f(v):
        v = F.pad(v, (r, r), mode="replicate")
        return F.max_pool1d(v, 2 * r + 1, stride=1) if is_max else -F.max_pool1d(-v, 2 * r + 1, stride=1)
    return _along(x, axis, f)


def box1d(x, axis, r):
    if r == 0:
        return x
    def f(v):
        v = F.pad(v, (r, r), mode="replicate")
        return F.avg_pool1d(v, 2 * r + 1, stride=1)
    return _along(x, axis, f)


def conv1d(x, axis, t):
    r = (t.numel() - 1) // 2
    return _along(x, axis, lambda v: F.conv1d(v, t.view(1, 1, -1), padding=r))


def normalize(I, rxy, rz, min_intensity):
    mn, mx = I, I
    for axis, r in ((2, rxy), (1, rxy), (0, rz)):
        mn = minmax1d(mn, axis, r, False)
        mx = minmax1d(mx, axis, r, True)
    e, d = mn, mx
    for axis, r in ((2, rxy), (1, rxy), (0, rz)):
        e = box1d(e, axis, r)
        d = box1d(d, axis, r)
    return torch.where(I >= min_intensity, (I - e) / (d - e), torch.zeros_like(I))


def gauss(x, sx, sy, sz):
    return conv1d(conv1d(conv1d(x, 2, taps(sx)), 1, taps(sy)), 0, taps(sz))


def dog(norm, sigma, gamma=1.0):
    sx1, sy1, sz1, sx2, sy2, sz2 = sigma
    return (gauss(norm, sx1, sy1, sz1) - gauss(norm, sx2, sy2, sz2)) * (sx1 * sy1 * sz1) ** gamma


def grad1(f, axis):
    """0.5 (f[+1] - f[-1]) with f = 0 outside the volume."""
    fp = F.pad(f.movedim(axis, -1), (1, 1))
    return (0.5 * (fp[..., 2:] - fp[..., :-2])).movedim(-1, axis)


def hessian(f):
    gx, gy, gz = grad1(f, 2), grad1(f, 1), grad1(f, 0)
    return [grad1(gx, 2), grad1(gx, 1), grad1(gx, 0), grad1(gy, 1), grad1(gy, 0), grad1(gz, 0)]


def soft_score(h, tau, b=(0.0, 0.0, 0.0)):
    """The three tests with thresholds b: xx < b0, xx yy - xy^2 > b1, det < b2 (b = 0: the
    reference's), each a sigmoid of its margin over tau, tau^2, tau^3."""
    xx, xy, xz, yy, yz, zz = h
    m2 = xx * yy - xy * xy
    det = xx * yy * zz + 2 * xy * yz * xz - xx * yz * yz - yy * xz * xz - zz * xy * xy
    return torch.sigmoid((b[0] - xx) / tau) * torch.sigmoid((m2 - b[1]) / tau ** 2) * \
        torch.sigmoid((b[2] - det) / tau ** 3)


def loss(I, sigma, pos, neg, rxy, rz, min_intensity, tau, gamma=1.0, b=(0.0, 0.0, 0.0)):
    """I: (D, H, W) float64; sigma: 6 float64 scalars (x1, y1, z1, x2, y2, z2); pos / neg:
    (n, 3) integer (z, y, x) voxel indices; b: the 3 test thresholds (float64 scalars)."""
    h = hessian(dog(normalize(I, rxy, rz, min_intensity), sigma, gamma))

    def at(p):
        return [e[p[:, 0], p[:, 1], p[:, 2]] for e in h]
    return soft_score(at(pos), tau, b).mean() - soft_score(at(neg), tau, b).mean()
