"""TEST INFRASTRUCTURE ONLY: runs the reference's own CUDA kernels on a GPU.

oracle/build_oracle.py compiles CUBIC-informatics src/3D/*.cu, unmodified, into
sm_103a cubins under oracle/_ref/.  This module loads them with the CUDA driver API
(ctypes on libcuda) and launches the kernels with the grid and block shapes the
reference's host wrappers use, in the same order, on the same buffer roles:
  Normalize3DFilter                    src/3D/NormalizeFilter.cu:537-654
  DoG3DFilter / initGaussian3DKernel   src/3D/DoG3DFilter.cu:132-437
  HessianPositiveDefiniteWithElement   src/3D/Hessian3DFilter_element.cu:76-388
  CCL                                  src/3D/CCL3D.cu:81-117
  Eigenvalues                          src/3D/Eigenvalues.cu:99-112
  Erosion3DFilter                      src/3D/Erosion3DFilter.cu:74-268
The reference kernels have no bounds checks, so every launch first checks the
divisibility and radius preconditions their host wrappers assert; shapes that fail
them raise ValueError before anything reaches the GPU.  Buffers are torch CUDA
tensors; torch's primary context is the one the modules load into.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
FILES = ["NormalizeFilter", "DoG3DFilter", "Hessian3DFilter_element", "CCL3D", "Eigenvalues", "Erosion3DFilter"]

_cu = None
_mods = {}
_funcs = {}


def available():
    return all(os.path.exists(os.path.join(REF_DIR, f + ".cubin")) for f in FILES)


def _drv():
    global _cu
    if _cu is None:
        _cu = ctypes.CDLL("libcuda.so.1")
    return _cu


def _ck(rc, what):
    if rc != 0:
        name = ctypes.c_char_p()
        _drv().cuGetErrorName(rc, ctypes.byref(name))
        raise RuntimeError("%s failed: %s (%d)" % (what, name.value, rc))


def _module(name):
    if name not in _mods:
        import torch
        torch.zeros(1, device="cuda")   # primary context current on this thread
        m = ctypes.c_void_p()
        _ck(_drv().cuModuleLoad(ctypes.byref(m), os.path.join(REF_DIR, name + ".cubin").encode()), "cuModuleLoad")
        _mods[name] = m
        cnt = ctypes.c_uint()
        _ck(_drv().cuModuleGetFunctionCount(ctypes.byref(cnt), m), "cuModuleGetFunctionCount")
        arr = (ctypes.c_void_p * cnt.value)()
        _ck(_drv().cuModuleEnumerateFunctions(arr, cnt, m), "cuModuleEnumerateFunctions")
        names = {}
        for f in arr:
            nm = ctypes.c_char_p()
            _ck(_drv().cuFuncGetName(ctypes.byref(nm), ctypes.c_void_p(f)), "cuFuncGetName")
            names[nm.value.decode()] = ctypes.c_void_p(f)
        _funcs[name] = names
    return _mods[name]


def _kernel(module, *parts):
    _module(module)
    hits = [f for n, f in _funcs[module].items() if all(p in n for p in parts)]
    if len(hits) != 1:
        raise RuntimeError("kernel %s in %s: %d matches" % (parts, module, len(hits)))
    return hits[0]


def _global(module, name):
    ptr = ctypes.c_uint64()
    size = ctypes.c_size_t()
    _ck(_drv().cuModuleGetGlobal_v2(ctypes.byref(ptr), ctypes.byref(size), _module(module), name.encode()),
        "cuModuleGetGlobal " + name)
    return ptr.value, size.value


def _launch(fn, grid, block, args):
    """args: list of ctypes values (c_uint64 for pointers, c_int, c_float)."""
    for g in grid:
        if g <= 0:
            raise ValueError("empty grid")
    holders = (ctypes.c_void_p * len(args))(*[ctypes.addressof(a) for a in args])
    _ck(_drv().cuLaunchKernel(fn, grid[0], grid[1], grid[2], block[0], block[1], block[2], 0, None, holders, None),
        "cuLaunchKernel")


def _sync():
    _ck(_drv().cuCtxSynchronize(), "cuCtxSynchronize")


def _p(t):
    return ctypes.c_uint64(t.data_ptr())


def _need(cond, msg):
    if not cond:
        raise ValueError("reference kernel precondition: " + msg)


# ---------------------------------------------------------------- normalization
def _norm_checks(W, H, D, rxy, rz):
    _need(W % 320 == 0 and H % 360 == 0 and D % 16 == 0, "W%320, H%360, D%16 (NormalizeFilter.cu:116-119,193-196,272-275)")
    _need(H % 2 == 0 and D % 2 == 0 and W % 8 == 0 and H % 8 == 0 and D % 8 == 0, "block divisibility")
    _need(rxy <= 256 and rxy <= 288 and rz <= 16, "radius within halo (rows 256, columns 288, layers 16)")


def normalize(img, rxy, rz, min_intensity):
    """Normalize3DFilter on a uint16 CUDA tensor (D, H, W) -> float32 tensor."""
    import torch
    D, H, W = img.shape
    norm = torch.empty((D, H, W), dtype=torch.float32, device=img.device)
    w, h, d = ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(D)
    if rxy == 0 or rz == 0:
        _need(W % 8 == 0 and H % 8 == 0 and D % 8 == 0, "8^3 blocks")
        _launch(_kernel("NormalizeFilter", "Copy3DKernel"), (W // 8, H // 8, D // 8), (8, 8, 8),
                [_p(img), _p(norm), ctypes.c_float(min_intensity), w, h, d])
        _sync()
        return norm
    _norm_checks(W, H, D, rxy, rz)
    tmp1 = torch.empty((D, H, W), dtype=torch.uint16, device=img.device)
    tmp2 = torch.empty((D, H, W), dtype=torch.uint16, device=img.device)
    ero_l = torch.empty((D, H, W), dtype=torch.float32, device=img.device)
    dil_l = torch.empty((D, H, W), dtype=torch.float32, device=img.device)
    R, RZ = ctypes.c_int(rxy), ctypes.c_int(rz)

    def minmax(is_min, dst, src):
        b = "Lb1E" if is_min else "Lb0E"
        _launch(_kernel("NormalizeFilter", "minmaxRows3DKernel", b), (W // 320, H // 2, D // 2), (64, 2, 2),
                [_p(dst), _p(src), w, h, d, R])
        _launch(_kernel("NormalizeFilter", "minmaxColumns3DKernel", b), (W // 2, H // 360, D // 2), (2, 72, 2),
                [_p(tmp1), _p(dst), w, h, d, R])
        _launch(_kernel("NormalizeFilter", "minmaxLayers3DKernel", b), (W // 8, H // 8, D // 16), (8, 8, 8),
                [_p(dst), _p(tmp1), w, h, d, RZ])

    def uniform(src_u16, result):
        _launch(_kernel("NormalizeFilter", "uniformRows3DKernel"), (W // 320, H // 2, D // 2), (64, 2, 2),
                [_p(result), _p(src_u16), w, h, d, R])
        _launch(_kernel("NormalizeFilter", "uniformColumns3DKernel"), (W // 2, H // 360, D // 2), (2, 72, 2),
                [_p(norm), _p(result), w, h, d, R])
        _launch(_kernel("NormalizeFilter", "uniformLayers3DKernel"), (W // 8, H // 8, D // 16), (8, 8, 8),
                [_p(result), _p(norm), w, h, d, RZ])

    minmax(True, tmp2, img)
    uniform(tmp2, ero_l)
    minmax(False, tmp2, img)
    uniform(tmp2, dil_l)
    _launch(_kernel("NormalizeFilter", "Normalize3DKernel"), (W // 8, H // 8, D // 8), (8, 8, 8),
            [_p(img), _p(ero_l), _p(dil_l), _p(norm), ctypes.c_float(min_intensity), w, h, d])
    _sync()
    return norm


# ---------------------------------------------------------------- DoG
def dog(norm, sigmas, taps_fn, normalizer):
    """DoG3DFilter.  sigmas = (xy_small, z_small, xy_large, z_large); taps_fn(sigma) ->
    (taps[80], radius) as initGaussian3DKernel builds them on the host; normalizer is
    the host powf product of DoG3DFilter.cu:432."""
    import torch
    D, H, W = norm.shape
    taps = np.zeros((4, 80), np.float32)
    radius = []
    for i, s in enumerate(sigmas):
        t, r = taps_fn(s)
        taps[i] = t
        radius.append(r)
    _need(W % 128 == 0 and H % 144 == 0 and D % 16 == 0 and H % 4 == 0 and D % 8 == 0 and W % 8 == 0,
          "W%128, H%144, D%16 (DoG3DFilter.cu:143,235,328)")
    _need(max(radius[0], radius[2]) <= 32 and max(radius[1], radius[3]) <= 8, "radius within halo (xy 32, z 8)")
    cptr, csize = _global("DoG3DFilter", "c_Kernel")
    _need(csize == taps.nbytes, "c_Kernel size")
    _ck(_drv().cuMemcpyHtoD_v2(ctypes.c_uint64(cptr), taps.ctypes.data, ctypes.c_size_t(taps.nbytes)), "c_Kernel upload")
    t1 = torch.empty_like(norm)
    t2 = torch.empty_like(norm)
    out = torch.empty_like(norm)
    w, h, d = ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(D)
    rows = _kernel("DoG3DFilter", "convolutionRows3DKernel")
    cols = _kernel("DoG3DFilter", "convolutionColumns3DKernel")
    lays = _kernel("DoG3DFilter", "convolutionLayers3DKernel")

    def gauss(result, kxy, kz):
        _launch(rows, (W // 128, H // 4, D // 4), (16, 4, 4),
                [_p(result), _p(norm), w, h, d, ctypes.c_int(kxy), ctypes.c_int(radius[kxy])])
        _launch(cols, (W // 4, H // 144, D // 4), (4, 16, 4),
                [_p(t1), _p(result), w, h, d, ctypes.c_int(kxy), ctypes.c_int(radius[kxy])])
        _launch(lays, (W // 8, H // 8, D // 16), (8, 8, 4),
                [_p(result), _p(t1), w, h, d, ctypes.c_int(kz), ctypes.c_int(radius[kz])])

    gauss(t2, 2, 3)
    gauss(out, 0, 1)
    _launch(_kernel("DoG3DFilter", "NormalizeSubtract3DKernel"), (W // 8, H // 8, D // 8), (8, 8, 8),
            [_p(out), _p(t2), w, h, d, ctypes.c_float(float(normalizer))])
    _sync()
    return out


# ---------------------------------------------------------------- Hessian + PD
def hessian_pd(dogv):
    """HessianPositiveDefiniteWithElement -> (hessian (6, D, H, W) float32, pd uint8)."""
    import torch
    D, H, W = dogv.shape
    _need(W % 128 == 0 and H % 144 == 0 and D % 8 == 0 and W % 8 == 0 and H % 8 == 0 and H % 4 == 0,
          "W%128, H%144, D%8 (Hessian3DFilter_element.cu:84-86,175-177,269-271)")
    hess = torch.empty((6, D, H, W), dtype=torch.float32, device=dogv.device)
    tmp = torch.empty_like(dogv)
    pd = torch.empty((D, H, W), dtype=torch.uint8, device=dogv.device)
    w, h, d = ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(D)
    rows = _kernel("Hessian3DFilter_element", "gradientRowsKernel")
    cols = _kernel("Hessian3DFilter_element", "gradientColumnsKernel")
    lays = _kernel("Hessian3DFilter_element", "gradientLayersKernel")

    def R(dst, src):
        _launch(rows, (W // 128, H // 4, D // 4), (16, 4, 4), [_p(dst), _p(src), w, h, d])

    def C(dst, src):
        _launch(cols, (W // 4, H // 144, D // 4), (4, 16, 4), [_p(dst), _p(src), w, h, d])

    def L(dst, src):
        _launch(lays, (W // 8, H // 8, D // 8), (8, 8, 4), [_p(dst), _p(src), w, h, d])

    R(tmp, dogv); R(hess[0], tmp); C(hess[1], tmp); L(hess[2], tmp)
    C(tmp, dogv); C(hess[3], tmp); L(hess[4], tmp)
    L(tmp, dogv); L(hess[5], tmp)
    _launch(_kernel("Hessian3DFilter_element", "PositiveDefiniteKernel"), (W // 8, H // 8, D // 8), (8, 8, 8),
            [_p(pd), _p(hess), w, h, d])
    _sync()
    return hess, pd


# ---------------------------------------------------------------- CCL
def ccl(pd, max_iterations=100000):
    """CCL: label-equivalence iterations until the device flag stays 0."""
    import torch
    D, H, W = pd.shape
    _need(W % 8 == 0 and H % 8 == 0 and D % 8 == 0, "8^3 blocks (CCL3D.cu:84-86)")
    labels = torch.empty((D, H, W), dtype=torch.int32, device=pd.device)
    w, h, d = ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(D)
    grid = (W // 8, H // 8, D // 8)
    _launch(_kernel("CCL3D", "initLabels"), grid, (8, 8, 8), [_p(pd), _p(labels), w, h, d])
    _sync()
    flag_ptr, _ = _global("CCL3D", "d_isNotDone")
    scan = _kernel("CCL3D", "scanLabels")
    analyse = _kernel("CCL3D", "analyseLabels")
    zero = ctypes.c_int(0)
    got = ctypes.c_int(0)
    for it in range(max_iterations):
        _ck(_drv().cuMemcpyHtoD_v2(ctypes.c_uint64(flag_ptr), ctypes.byref(zero), ctypes.c_size_t(4)), "flag reset")
        _launch(scan, grid, (8, 8, 8), [_p(labels), w, h, d])
        _sync()
        _ck(_drv().cuMemcpyDtoH_v2(ctypes.byref(got), ctypes.c_uint64(flag_ptr), ctypes.c_size_t(4)), "flag read")
        if not got.value:
            return labels, it + 1
        _launch(analyse, grid, (8, 8, 8), [_p(labels), w, h, d])
        _sync()
    raise RuntimeError("reference CCL did not converge in %d iterations" % max_iterations)


# ---------------------------------------------------------------- eigen features
def eigen(hess_sums):
    """EigenvaluesKernel<float> on region sums (6, R) float32 -> (structureness, blobness)."""
    import torch
    R = hess_sums.shape[1]
    pitch = R
    src = torch.as_tensor(np.ascontiguousarray(hess_sums, np.float32).reshape(-1)).cuda()
    # three planes: the zero-matrix branch also writes the third one (Eigenvalues.cu:43-49)
    dst = torch.zeros(3 * pitch, dtype=torch.float32, device="cuda")
    _launch(_kernel("Eigenvalues", "EigenvaluesKernel"), (R, 1, 1), (1, 1, 1),
            [_p(src), _p(dst), ctypes.c_int(R), ctypes.c_int(pitch)])
    _sync()
    out = dst.cpu().numpy()
    return out[:R], out[pitch:2 * pitch]


# ---------------------------------------------------------------- erosion
def erosion(img, rxy, rz):
    """Erosion3DFilter (zero border) on a uint16 CUDA tensor."""
    import torch
    D, H, W = img.shape
    _need(W % 128 == 0 and H % 144 == 0 and D % 8 == 0 and H % 4 == 0 and D % 4 == 0,
          "W%128, H%144, D%8 (Erosion3DFilter.cu:80-85,173-176,245-248)")
    _need(rxy <= 16 and rz <= 8, "radius within halo (xy 16, z 8)")
    tmp = torch.empty_like(img)
    out = torch.empty_like(img)
    w, h, d = ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(D)
    _launch(_kernel("Erosion3DFilter", "erosionRows3DKernel"), (W // 128, H // 4, D // 4), (16, 4, 4),
            [_p(out), _p(img), w, h, d, ctypes.c_int(rxy)])
    _launch(_kernel("Erosion3DFilter", "erosionColumns3DKernel"), (W // 4, H // 144, D // 4), (4, 16, 4),
            [_p(tmp), _p(out), w, h, d, ctypes.c_int(rxy)])
    _launch(_kernel("Erosion3DFilter", "erosionLayers3DKernel"), (W // 8, H // 8, D // 8), (8, 8, 4),
            [_p(out), _p(tmp), w, h, d, ctypes.c_int(rz)])
    _sync()
    return out
