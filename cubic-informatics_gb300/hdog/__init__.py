"""Python host interface of the GB300 HDoG library (ctypes over include/hdog.h).

Mirrors the reference's host functions for the HDoG path (CUBIC-informatics src/3D):
Normalize3DFilter, DoG3DFilter, HessianPositiveDefiniteWithElement, CCL, the regional
feature reductions, Erosion3DFilter, processSubstack and the HDoG3D_main executable.
Device buffers are torch CUDA tensors; records come back as numpy arrays of the
reference's ``dt_local`` layout (script/HalfBrainCells.py:11-15).

The CUDA library must be built (``build()``); nothing here falls back to a CPU path.
"""
import ctypes
import json
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)
BUILD_DIR = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libhdog.so")
SYNTH_PATH = os.path.join(BUILD_DIR, "libhdog_synth.so")
MAIN_PATH = os.path.join(BUILD_DIR, "hdog_main")

HDOG_OK, HDOG_ERR_ARG, HDOG_ERR_SHAPE, HDOG_ERR_CUDA, HDOG_ERR_IO = 0, 1, 2, 3, 4
HDOG_ERR_PARAM, HDOG_ERR_CAPACITY, HDOG_ERR_TIMEOUT, HDOG_ERR_NOMEM = 5, 6, 7, 8
HDOG_OPT_FUSED_SWEEP, HDOG_OPT_HOST_BATCH, HDOG_OPT_WALK_LIMIT = 1, 2, 3

# The 28-byte candidate record (FeatureVector, src/3D/utils.h:188-197).
DT_LOCAL = np.dtype([
    ("local_x", "<f4"), ("local_y", "<f4"), ("local_z", "<f4"),
    ("structureness", "<f4"), ("blobness", "<f4"), ("intensity", "<f4"),
    ("size", "<u2"), ("padding", "<u2"),
])


class HDoGError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("hdog error %d: %s" % (code, message))
        self.code = code


class hdog_params(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int), ("depth", ctypes.c_int),
        ("left_margin", ctypes.c_int), ("right_margin", ctypes.c_int),
        ("top_margin", ctypes.c_int), ("bottom_margin", ctypes.c_int),
        ("extra_depth_margin", ctypes.c_int),
        ("radius_norm_xy", ctypes.c_int), ("radius_norm_z", ctypes.c_int),
        ("min_intensity", ctypes.c_int),
        ("gamma_n", ctypes.c_float),
        ("sigma_xy_small", ctypes.c_float), ("sigma_z_small", ctypes.c_float),
        ("sigma_xy_large", ctypes.c_float), ("sigma_z_large", ctypes.c_float),
        ("min_size", ctypes.c_int), ("is_ave_mode", ctypes.c_int),
        ("erosion_radius_xy", ctypes.c_int), ("erosion_radius_z", ctypes.c_int),
        ("dev_id", ctypes.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class hdog_regions(ctypes.Structure):
    _fields_ = [
        ("num_regions", ctypes.c_int64),
        ("label", ctypes.c_void_p), ("count", ctypes.c_void_p), ("intensity", ctypes.c_void_p),
        ("centroid", ctypes.c_void_p), ("hessian", ctypes.c_void_p), ("eigen", ctypes.c_void_p),
        ("pitch", ctypes.c_int64),
    ]


_P = ctypes.c_void_p
HDOG_PROMOTE_F32, HDOG_PROMOTE_F64 = 0, 1

# dt_global (script/HalfBrainCells.py:16-20) and dt_scalemerged (script/MergeBrain.py:32-35)
DT_GLOBAL = np.dtype([("merged_x", "f4"), ("merged_y", "f4"), ("merged_z", "f4"),
                      ("i_x", "u1"), ("i_y", "u1"), ("FWRV", "u1")])
DT_SCALEMERGED = np.dtype([("scaled_x", "f4"), ("scaled_y", "f4"), ("scaled_z", "f4"), ("is_valid", "bool")])


class hdog_global_params(ctypes.Structure):
    _fields_ = [("offset_x", ctypes.c_double), ("offset_y", ctypes.c_double), ("offset_z", ctypes.c_double),
                ("scale_x", ctypes.c_double), ("scale_y", ctypes.c_double), ("scale_z", ctypes.c_double),
                ("width", ctypes.c_int), ("height", ctypes.c_int), ("is_fw", ctypes.c_int),
                ("i_x", ctypes.c_int), ("i_y", ctypes.c_int), ("promote", ctypes.c_int)]


class hdog_scalemerge_params(ctypes.Structure):
    _fields_ = [("bound_z0", ctypes.c_double), ("bound_z1", ctypes.c_double),
                ("offset_x", ctypes.c_double), ("offset_y", ctypes.c_double), ("offset_z", ctypes.c_double),
                ("coeff_x", ctypes.c_double), ("coeff_y", ctypes.c_double), ("coeff_z", ctypes.c_double),
                ("margin_left", ctypes.c_double), ("margin_top", ctypes.c_double),
                ("A", ctypes.c_double * 9), ("b", ctypes.c_double * 3), ("promote", ctypes.c_int)]


class hdog_clf_params(ctypes.Structure):
    _fields_ = [("bias", ctypes.c_double * 3), ("scale", ctypes.c_double * 3),
                ("bias_before_log", ctypes.c_double * 3), ("is_ave", ctypes.c_int)]


class hdog_stack_in(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("on_device", ctypes.c_int), ("length", ctypes.c_int)]


class hdog_graph_stack(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("width", ctypes.c_int), ("height", ctypes.c_int), ("length", ctypes.c_int)]


class hdog_soft_params(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int), ("depth", ctypes.c_int),
                ("radius_norm_xy", ctypes.c_int), ("radius_norm_z", ctypes.c_int),
                ("min_intensity", ctypes.c_float), ("sigma", ctypes.c_float * 6), ("gamma", ctypes.c_float),
                ("tau", ctypes.c_float), ("thresh", ctypes.c_float * 3)]


_SIGNATURES = {
    "hdog_last_error": (ctypes.c_char_p, []),
    "hdog_abi_version": (ctypes.c_int, []),
    "hdog_params_load_json": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(hdog_params)]),
    "hdog_gaussian_taps": (ctypes.c_int, [ctypes.c_float, _P, ctypes.POINTER(ctypes.c_int)]),
    "hdog_depth_margin": (ctypes.c_int, [ctypes.POINTER(hdog_params), ctypes.POINTER(ctypes.c_int)]),
    "hdog_ctx_create": (ctypes.c_int, [ctypes.POINTER(hdog_params), ctypes.c_int, ctypes.POINTER(_P)]),
    "hdog_ctx_destroy": (ctypes.c_int, [_P]),
    "hdog_ctx_bytes": (ctypes.c_int, [ctypes.POINTER(hdog_params), ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "hdog_normalize": (ctypes.c_int, [_P, _P, _P, _P]),
    "hdog_normalize_parts": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "hdog_dog": (ctypes.c_int, [_P, _P, _P, _P]),
    "hdog_hessian_pd": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "hdog_ccl": (ctypes.c_int, [_P, _P, _P, _P]),
    "hdog_regional_features": (ctypes.c_int, [_P, _P, _P, _P, ctypes.POINTER(hdog_regions), _P]),
    "hdog_erosion": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, _P]),
    "hdog_run_substack": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int64,
                                         ctypes.POINTER(ctypes.c_int64), _P]),
    "hdog_run_stack": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int64,
                                      ctypes.POINTER(ctypes.c_int64), _P]),
    "hdog_last_records": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "hdog_run_stacks": (ctypes.c_int, [_P, ctypes.POINTER(hdog_stack_in), ctypes.c_int, _P, ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_int64), _P, _P]),
    "hdog_run_param_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int]),
    "hdog_graph_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.POINTER(hdog_graph_stack), ctypes.c_int,
                                         _P, ctypes.POINTER(_P)]),
    "hdog_graph_run": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64), _P, _P]),
    "hdog_graph_last_records": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]),
    "hdog_graph_destroy": (ctypes.c_int, [_P]),
    "hdog_autotune": (ctypes.c_int, [_P, _P, ctypes.c_int, _P]),
    "hdog_ctx_tuning": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "hdog_ctx_set_option": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "hdog_ccl_noalloc": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]),
    "hdog_ccl_edge_count": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "hdog_timing_enable": (ctypes.c_int, [_P, ctypes.c_int]),
    "hdog_timing_read": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "hdog_records_to_global": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(hdog_global_params), _P, _P]),
    "hdog_scale_merge": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(hdog_scalemerge_params), _P, _P]),
    "hdog_classifier_features": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(hdog_clf_params), _P, _P]),
    "hdog_soft_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(hdog_soft_params)]),
    "hdog_soft_forward": (ctypes.c_int, [ctypes.POINTER(hdog_soft_params), _P, _P, ctypes.c_int, _P, ctypes.c_int,
                                         _P, _P, _P, _P]),
    "hdog_soft_backward": (ctypes.c_int, [ctypes.POINTER(hdog_soft_params), _P, _P, ctypes.c_int, _P, ctypes.c_int,
                                          ctypes.c_float, _P, _P, _P, _P, _P]),
    "hdog_soft_backward_kept": (ctypes.c_int, [ctypes.POINTER(hdog_soft_params), _P, _P, ctypes.c_int, _P,
                                               ctypes.c_int, ctypes.c_float, _P, _P, _P, _P, _P]),
    "hdog_memcpy": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "hdog_stream_sync": (ctypes.c_int, [_P]),
    "hdog_device_alloc": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_size_t]),
    "hdog_device_free": (ctypes.c_int, [_P]),
}

_lib = None


def lib():
    """The loaded libhdog.so; raises when the CUDA library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise HDoGError(HDOG_ERR_ARG, "libhdog.so is not built (%s); run build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def build(verbose=False):
    import importlib.util
    spec = importlib.util.spec_from_file_location("_hdog_build", os.path.join(_PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose)


def check(rc):
    if rc != HDOG_OK:
        raise HDoGError(rc, lib().hdog_last_error().decode("utf-8", "replace"))


# ---------------------------------------------------------------- parameters
PARAM_DEFAULTS = dict(width=2560, height=2160, depth=32, left_margin=100, right_margin=100, top_margin=100,
                      bottom_margin=100, extra_depth_margin=3, radius_norm_xy=100, radius_norm_z=5,
                      min_intensity=1000, gamma_n=1.0, sigma_xy_small=4.0, sigma_z_small=1.8,
                      sigma_xy_large=6.0, sigma_z_large=2.7, min_size=10, is_ave_mode=0,
                      erosion_radius_xy=0, erosion_radius_z=0, dev_id=0)


def make_params(**kw):
    p = hdog_params()
    d = dict(PARAM_DEFAULTS)
    d.update(kw)
    for k, v in d.items():
        setattr(p, k, v)
    return p


def load_param_file(path):
    """loadParamFile (src/3D/utils.h:95-157): the HDoG keys of a parameter JSON."""
    p = hdog_params()
    check(lib().hdog_params_load_json(os.fsencode(path), ctypes.byref(p)))
    return p


def write_param_file(path, p, stacks, gpus=(0,)):
    """Writes a parameter JSON in the reference's layout (param/param_example_HDoG_FW.json)
    with `stacks` = [(dst_path, [src_path, ...]), ...]."""
    d = {
        "devID": int(p.dev_id), "gpus": list(gpus),
        "input_image_info": {"width": p.width, "height": p.height, "left_margin": p.left_margin,
                             "right_margin": p.right_margin, "top_margin": p.top_margin,
                             "bottom_margin": p.bottom_margin},
        "coordinate_info": {"scale_x": 1.0, "scale_y": 1.0, "scale_z": 1.0},
        "HDoG_param": {"depth": p.depth, "extra_depth_margin": p.extra_depth_margin,
                       "radius_norm": {"xy_large": p.radius_norm_xy, "z_large": p.radius_norm_z},
                       "min_intensity": p.min_intensity, "gamma_n": p.gamma_n,
                       "sigma_dog": {"xy_small": p.sigma_xy_small, "z_small": p.sigma_z_small,
                                     "xy_large": p.sigma_xy_large, "z_large": p.sigma_z_large},
                       "min_size": p.min_size},
        "is_ave_mode": bool(p.is_ave_mode),
        "stacks": [{"dst_path": dst, "src_paths": list(src)} for dst, src in stacks],
    }
    if p.erosion_radius_xy or p.erosion_radius_z:
        d["HDoG_param"]["erosion_radius"] = {"xy": p.erosion_radius_xy, "z": p.erosion_radius_z}
    with open(path, "w") as f:
        json.dump(d, f, indent=2)


def gaussian_taps(sigma):
    """calcGaussianWeight (src/3D/DoG3DFilter.cu:372-392) -> (taps[80] float32, radius)."""
    taps = np.zeros(80, np.float32)
    r = ctypes.c_int()
    check(lib().hdog_gaussian_taps(ctypes.c_float(sigma), taps.ctypes.data, ctypes.byref(r)))
    return taps, r.value


def depth_margin(p):
    m = ctypes.c_int()
    check(lib().hdog_depth_margin(ctypes.byref(p), ctypes.byref(m)))
    return m.value


def substack_schedule(length, depth, margin):
    """z0 of each substack (src/3D/HDoG3D_main.cpp:309-314)."""
    if length - margin <= 0:
        return []
    stride = depth - 2 * margin
    if stride <= 0:
        raise HDoGError(HDOG_ERR_PARAM, "depth must exceed twice the depth margin")
    return list(range(0, length - margin, stride))


def run_param_file(path, verbose=False):
    """The HDoG3D_main executable as a call (src/3D/HDoG3D_main.cpp:260-319)."""
    check(lib().hdog_run_param_file(os.fsencode(path), int(bool(verbose))))


# ---------------------------------------------------------------- device context
def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


class Context:
    """Device scratch for up to `max_substacks` substacks of width x height x depth.

    Stage methods take and return torch CUDA tensors shaped (depth, height, width),
    x fastest, as the reference's device buffers."""

    def __init__(self, params, max_substacks=1):
        self.params = params
        h = ctypes.c_void_p()
        check(lib().hdog_ctx_create(ctypes.byref(params), int(max_substacks), ctypes.byref(h)))
        self._h = h
        self.max_substacks = max_substacks

    def close(self):
        if self._h:
            lib().hdog_ctx_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def shape(self):
        p = self.params
        return (p.depth, p.height, p.width)

    def _empty(self, dtype):
        import torch
        return torch.empty(self.shape, dtype=dtype, device="cuda:%d" % self.params.dev_id)

    def set_fused_sweep(self, on):
        """DoG + Hessian + PD in one z-sweep kernel (default) or as separate passes."""
        check(lib().hdog_ctx_set_option(self._h, HDOG_OPT_FUSED_SWEEP, int(bool(on))))

    def set_host_batch(self, n):
        """Substacks in the first batch of run_stack with a host-memory stack (0: the
        context's max_substacks); the copy of the later slices overlaps that batch."""
        check(lib().hdog_ctx_set_option(self._h, HDOG_OPT_HOST_BATCH, int(n)))

    def ccl_edge_count(self):
        """(edges, capacity) of the last labelling's first substack: cross-tile edges found
        and the edge list's size (more edges than that are merged from the mask)."""
        e, c = ctypes.c_int64(), ctypes.c_int64()
        check(lib().hdog_ccl_edge_count(self._h, ctypes.byref(e), ctypes.byref(c)))
        return e.value, c.value

    def set_walk_limit(self, n):
        """Bound of the labelling's union-find walks (0: the default, no walk reaches it); a
        walk past it makes the call raise HDoGError with HDOG_ERR_TIMEOUT."""
        check(lib().hdog_ctx_set_option(self._h, HDOG_OPT_WALK_LIMIT, int(n)))

    def timing(self, on=True):
        """Per-kernel CUDA-event timing of this context's launches."""
        check(lib().hdog_timing_enable(self._h, int(bool(on))))

    def timing_read(self):
        """{kernel: (launches, total_ms)} since the last read ({} when timing is off)."""
        buf = ctypes.create_string_buffer(1 << 16)
        check(lib().hdog_timing_read(self._h, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split()
            out[name] = (int(cnt), float(ms))
        return out

    # Normalize3DFilter (src/3D/NormalizeFilter.cu:603-654)
    def normalize(self, img, out=None, stream=None):
        import torch
        assert img.dtype == torch.uint16 and img.is_cuda and img.is_contiguous()
        out = self._empty(torch.float32) if out is None else out
        check(lib().hdog_normalize(self._h, _ptr(img), _ptr(out), _stream(stream)))
        return out

    def normalize_parts(self, img, stream=None):
        """(norm, erosion_l, dilation_l): the normalized volume and the box means of the
        min and the max it divides by (test/Normalize_test.cpp dumps all three)."""
        import torch
        assert img.dtype == torch.uint16 and img.is_cuda and img.is_contiguous()
        norm, ero, dil = (self._empty(torch.float32) for _ in range(3))
        check(lib().hdog_normalize_parts(self._h, _ptr(img), _ptr(norm), _ptr(ero), _ptr(dil), _stream(stream)))
        return norm, ero, dil

    # DoG3DFilter (src/3D/DoG3DFilter.cu:431-437)
    def dog(self, norm, out=None, stream=None):
        import torch
        out = self._empty(torch.float32) if out is None else out
        check(lib().hdog_dog(self._h, _ptr(norm), _ptr(out), _stream(stream)))
        return out

    # HessianPositiveDefiniteWithElement (src/3D/Hessian3DFilter_element.cu:355-388)
    def hessian_pd(self, dog, want_hessian=False, stream=None):
        import torch
        mask = self._empty(torch.uint8)
        hess = None
        if want_hessian:
            hess = torch.empty((6,) + self.shape, dtype=torch.float32, device=dog.device)
        check(lib().hdog_hessian_pd(self._h, _ptr(dog), _ptr(mask), _ptr(hess) if hess is not None else None,
                                    _stream(stream)))
        return mask, hess

    # CCL (src/3D/CCL3D.cu:81-117)
    def ccl(self, mask, stream=None):
        import torch
        labels = self._empty(torch.int32)
        check(lib().hdog_ccl(self._h, _ptr(mask), _ptr(labels), _stream(stream)))
        return labels

    # HessianFeatures + Eigenvalues + MaxNormalized/SumNormalized + RegionalSizeAndCentroid
    def regional_features(self, labels, norm, dog, stream=None):
        """Per-region arrays (region 0 = background), ordered by label, as numpy."""
        r = hdog_regions()
        check(lib().hdog_regional_features(self._h, _ptr(labels), _ptr(norm), _ptr(dog), ctypes.byref(r),
                                           _stream(stream)))
        n = int(r.num_regions)
        cap = int(r.pitch)

        def fetch(ptr, dtype, rows=1):
            out = np.empty((rows, n), dtype)
            for k in range(rows):
                src = ptr + k * cap * np.dtype(dtype).itemsize
                check(lib().hdog_memcpy(out[k].ctypes.data, ctypes.c_void_p(src), n * np.dtype(dtype).itemsize, None))
            return out if rows > 1 else out[0]

        return {
            "num_regions": n,
            "label": fetch(r.label, np.int32),
            "count": fetch(r.count, np.uint32),
            "intensity": fetch(r.intensity, np.float32),
            "centroid": fetch(r.centroid, np.float32, 3),
            "hessian": fetch(r.hessian, np.float32, 6),
            "eigen": fetch(r.eigen, np.float32, 2),
        }

    # Erosion3DFilter (src/3D/Erosion3DFilter.cu:260-268)
    def erosion(self, src, radius_xy, radius_z, stream=None):
        import torch
        out = self._empty(torch.uint16)
        check(lib().hdog_erosion(self._h, _ptr(src), _ptr(out), int(radius_xy), int(radius_z), _stream(stream)))
        return out

    # processSubstack + saveFeatureVector
    def run_substack(self, img, depth_valid, z0, cap=None, stream=None, out=None):
        """img: host numpy uint16 (depth_valid, H, W) or a CUDA tensor; -> dt_local records.
        out: an optional dt_local array to fill (the result is then a view of it, or a
        new array when it is too small)."""
        on_dev, ptr = _buffer(img)
        out = _out_array(out, cap)
        n = ctypes.c_int64()
        rc = lib().hdog_run_substack(self._h, ptr, on_dev, int(depth_valid), int(z0), _out_ptr(out), len(out),
                                     ctypes.byref(n), _stream(stream) if on_dev else None)
        return self._finish(rc, out, n)

    def run_stack(self, stack, cap=None, stream=None, out=None):
        """All substacks of one stack (length, H, W) in the reference's schedule.  out: an
        optional dt_local array to fill, as for run_substack (reusing one array across calls
        saves mapping fresh pages for every result; in page-locked memory, e.g. a view of a
        pinned torch tensor, the records are copied into it straight from the device)."""
        on_dev, ptr = _buffer(stack)
        length = int(stack.shape[0])
        out = _out_array(out, cap)
        n = ctypes.c_int64()
        rc = lib().hdog_run_stack(self._h, ptr, on_dev, length, _out_ptr(out), len(out), ctypes.byref(n),
                                  _stream(stream) if on_dev else None)
        return self._finish(rc, out, n)

    def run_stacks(self, stacks, cap=None, stream=None, out=None):
        """Many stacks (each (length, H, W): numpy uint16 or CUDA tensor) with their
        substacks packed into full batches across stacks -> (records, per-stack counts);
        the records are stack by stack, as run_stack gives each stack's."""
        descs = (hdog_stack_in * max(1, len(stacks)))()
        for i, a in enumerate(stacks):
            on_dev, ptr = _buffer(a)
            descs[i].data = ptr.value
            descs[i].on_device = on_dev
            descs[i].length = int(a.shape[0])
        counts = np.zeros(max(1, len(stacks)), np.int64)
        out = _out_array(out, cap)
        n = ctypes.c_int64()
        rc = lib().hdog_run_stacks(self._h, descs, len(stacks), _out_ptr(out), len(out), ctypes.byref(n),
                                   ctypes.c_void_p(counts.ctypes.data), _stream(stream))
        return self._finish(rc, out, n), counts[:len(stacks)]

    def autotune(self, stack, stream=None):
        """Picks the sweeps' launch shapes and the substacks per launch of the graph form by
        timing this context's first batch of `stack` (a CUDA tensor (length, H, W))."""
        assert stack.is_cuda and stack.is_contiguous()
        check(lib().hdog_autotune(self._h, _ptr(stack), int(stack.shape[0]), _stream(stream)))
        return self.tuning()

    def tuning(self):
        """The autotuner's choice and timings for this context ({} before it ran)."""
        buf = ctypes.create_string_buffer(4096)
        check(lib().hdog_ctx_tuning(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def _finish(self, rc, out, n):
        """Records of a whole-chain call.  Without a capacity the call only counts them, and
        one copy from the context's host copy of the result fills an array of exactly that
        size; a buffer that was too small is refilled the same way, without running the chain
        again."""
        if rc == HDOG_ERR_CAPACITY:
            out = np.empty(int(n.value), DT_LOCAL)
            rc = lib().hdog_last_records(self._h, _out_ptr(out), len(out), ctypes.byref(n))
        check(rc)
        return out[: n.value]


class Graph:
    """The batched graph form: stacks of uneven depth and frame shape (CUDA tensors
    (length, H, W)) through one captured CUDA graph, one context per frame shape.
    run() -> (records stack by stack in the given order, per-stack counts)."""

    def __init__(self, contexts, stacks, stream=None):
        self._stacks = list(stacks)          # the graph keeps their device addresses
        self.contexts = list(contexts)
        ctxs = (ctypes.c_void_p * len(self.contexts))(*[c._h.value for c in self.contexts])
        descs = (hdog_graph_stack * max(1, len(self._stacks)))()
        for i, a in enumerate(self._stacks):
            assert a.is_cuda and a.is_contiguous() and a.dim() == 3
            descs[i].data = a.data_ptr()
            descs[i].length, descs[i].height, descs[i].width = (int(x) for x in a.shape)
        h = ctypes.c_void_p()
        check(lib().hdog_graph_create(ctxs, len(self.contexts), descs, len(self._stacks), _stream(stream),
                                      ctypes.byref(h)))
        self._h = h

    def run(self, cap=None, stream=None, out=None):
        out = _out_array(out, cap)
        counts = np.zeros(max(1, len(self._stacks)), np.int64)
        n = ctypes.c_int64()
        rc = lib().hdog_graph_run(self._h, _out_ptr(out), len(out), ctypes.byref(n),
                                  ctypes.c_void_p(counts.ctypes.data), _stream(stream))
        if rc == HDOG_ERR_CAPACITY:
            out = np.empty(int(n.value), DT_LOCAL)
            rc = lib().hdog_graph_last_records(self._h, _out_ptr(out), len(out), ctypes.byref(n))
        check(rc)
        return out[: n.value], counts[:len(self._stacks)]

    def close(self):
        if getattr(self, "_h", None):
            lib().hdog_graph_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _out_ptr(a):
    return a.ctypes.data if len(a) else None


def _out_array(out, cap):
    if out is None:
        return np.empty(cap or 0, DT_LOCAL)
    assert out.dtype == DT_LOCAL and out.ndim == 1 and out.flags["C_CONTIGUOUS"]
    return out


def _buffer(a):
    if isinstance(a, np.ndarray):
        assert a.dtype == np.uint16 and a.flags["C_CONTIGUOUS"]
        return 0, ctypes.c_void_p(a.ctypes.data)
    assert a.is_cuda and a.is_contiguous()
    return 1, ctypes.c_void_p(a.data_ptr())


from . import synth  # noqa: E402,F401
from .postprocess import records_to_global, scale_merge, classifier_features  # noqa: E402,F401
from . import soft  # noqa: E402,F401
