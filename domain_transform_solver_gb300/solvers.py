"""Python mirror of the reference's solver classes over libdtsgb's C ABI.

Class, method and argument names follow the reference C++ API
(src/domain_transform_filter.h, src/domain_transform_solver.h, src/hfbs.h,
src/edge_aware_solver.h) so a user of the reference finds the same calls:

    solver = DomainTransformSolver(ImageDim(640, 480))
    solver.SetImageDim(ImageDim(640, 480))
    solver.ClearAll()
    solver.InitFrame(COLOR_SPACE.YCbCr, rgba, target, confidence)
    solver.ComputeColorSpaceDifferential(DomainFilterParams(8, 8, 0.1))
    solver.IntegrateColorDifferentials()
    solver.Optimize(DomainOptimizeParams(num_iterations=10, ...))
    out = solver.Download(ImageType.OPTIMIZED_QUANTITY)

Images are numpy arrays: RGBA uint8 (H, W, 4) and float32 (H, W).  Errors
raise DtsgbError instead of printing; the HFBS "grid too large" case warns
and copies the target to the output, like the reference.
"""
from __future__ import annotations

import ctypes
import enum
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (ConfParams, DtsgbError, FilterParams, HfbsParams,
                   OptimizeParams, check)

__all__ = [
    "ImageDim", "ImageType", "COLOR_SPACE", "RobustLoss", "DomainFilterParams",
    "DomainFilterParamsVec1", "DomainOptimizeParams", "HFBSGridParams",
    "DomainTransformFilter", "DomainTransformSolver", "HFBS", "DtsOptions",
    "HfbsOptions", "Solve", "EdgeAwareOptimize", "DtsgbError", "SoftDTS",
    "FLAG_BF16_STORAGE", "FLAG_FIX_Y_LIMIT", "TUNE_DTS_TILE", "TUNE_HFBS_GROUP_VOXELS",
    "TUNE_REUSE_GUIDE_STATE", "TUNE_HFBS_SOLVE_STEPS", "TUNE_BOUNDS_SEGMENT",
    "Batch", "Pipeline", "DomainTransformStereo",
]

FLAG_BF16_STORAGE = 0x1
FLAG_FIX_Y_LIMIT = 0x2
FLAG_FILTER_ONLY = 0x4
FLAG_STEREO = 0x8
TUNE_DTS_TILE = 0
TUNE_HFBS_GROUP_VOXELS = 1
TUNE_REUSE_GUIDE_STATE = 2
TUNE_HFBS_SOLVE_STEPS = 3
TUNE_BOUNDS_SEGMENT = 4
# knob -> name, for reports
TUNE_NAMES = {TUNE_DTS_TILE: "dts_tile", TUNE_HFBS_GROUP_VOXELS: "hfbs_group_voxels",
              TUNE_REUSE_GUIDE_STATE: "reuse_guide_state",
              TUNE_HFBS_SOLVE_STEPS: "hfbs_solve_steps",
              TUNE_BOUNDS_SEGMENT: "bounds_segment"}


@dataclass
class ImageDim:  # src/domain_transform_common.h:7-17
    width: int = 100
    height: int = 200

    def Transpose(self) -> "ImageDim":
        return ImageDim(self.height, self.width)


class ImageType(enum.IntEnum):  # src/domain_transform_common.h:20-28
    COLOR_IMAGE = 0
    DIFFERENTIAL = 1
    INTEGRAL = 2
    TARGET = 3
    CONFIDENCE = 4
    OPTIMIZED_QUANTITY = 5
    TEST = 6


class COLOR_SPACE(enum.IntEnum):  # src/domain_transform_common.h:32
    RGB = 0
    YCbCr = 1
    YYY = 2


class RobustLoss(enum.IntEnum):  # src/domain_transform_optimize.h:8
    L1 = 0
    L2 = 1
    CHARBONNIER = 2


@dataclass
class DomainFilterParams:  # DomainFilterParamsVec<0>, filter_params.h:8-27
    sigma_x: float = 8.0
    sigma_y: float = 8.0
    sigma_r: float = 0.2

    def _c(self) -> FilterParams:
        return FilterParams(self.sigma_x, self.sigma_y, self.sigma_r)


@dataclass
class DomainFilterParamsVec1:  # DomainFilterParamsVec<1>
    sigma_x: float = 8.0
    sigma_y: float = 8.0
    sigma_r: float = 0.2
    sigmas: list = field(default_factory=lambda: [16.0, 0.0])

    def _c(self) -> ConfParams:
        s = list(self.sigmas) + [0.0, 0.0]
        return ConfParams(self.sigma_x, self.sigma_y, self.sigma_r,
                          (ctypes.c_float * 2)(s[0], s[1]))


@dataclass
class DomainOptimizeParams:  # src/domain_transform_optimize.h:29-50
    num_iterations: int = 3
    loss: RobustLoss = RobustLoss.L2
    lambda_: float = 1.0
    sigma_z: float = 100.0
    step_size: float = 0.99
    photo_consis_lambda: float = 1.0
    DT_lambda: float = 0.2

    def _c(self) -> OptimizeParams:
        return OptimizeParams(int(self.num_iterations), int(self.loss),
                              self.lambda_, self.sigma_z, self.step_size,
                              self.photo_consis_lambda, self.DT_lambda)


@dataclass
class HFBSGridParams:  # src/hfbs.h:18-60
    sigma_x: float = 8.0
    sigma_y: float = 8.0
    sigma_l: float = 4.0
    lambda_: float = 8.0
    alpha: float = 1.0
    beta: float = 0.9
    bistoch_iter_max: int = 20
    optim_iter_max: int = 140
    neg_exp_beta: float = 0.9
    grid_x: int = 1
    grid_y: int = 1
    grid_l: int = 1

    def _c(self) -> HfbsParams:
        return HfbsParams(self.sigma_x, self.sigma_y, self.sigma_l,
                          self.lambda_, self.alpha, self.beta,
                          int(self.bistoch_iter_max), int(self.optim_iter_max),
                          self.neg_exp_beta, self.grid_x, self.grid_y,
                          self.grid_l)


def _ptr(a) -> ctypes.c_void_p | None:
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)


def _f32(a, shape) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.size != shape[0] * shape[1]:
        raise ValueError(f"expected {shape[0]}x{shape[1]} floats, got {a.shape}")
    return a


def _rgba(a, shape) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint8)
    if a.size != shape[0] * shape[1] * 4:
        raise ValueError(f"expected {shape[0]}x{shape[1]}x4 bytes, got {a.shape}")
    return a


class DomainTransformFilter:
    """src/domain_transform_filter.h:19-70."""

    _flags_base = FLAG_FILTER_ONLY

    def __init__(self, max_image_dims: ImageDim, flags: int = 0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.dtsgb_dts_create(max_image_dims.width,
                                         max_image_dims.height,
                                         flags | self._flags_base,
                                         ctypes.byref(h)))
        self._h = h
        self.max_image_dims_ = ImageDim(max_image_dims.width, max_image_dims.height)
        self.image_dims_ = ImageDim(max_image_dims.width, max_image_dims.height)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dtsgb_dts_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def SetStream(self, stream_handle: int | None) -> None:
        check(self._lib.dtsgb_dts_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def SetImageDim(self, image_dim: ImageDim) -> None:
        check(self._lib.dtsgb_dts_set_image_dim(self._h, image_dim.width,
                                                image_dim.height))
        self.image_dims_ = ImageDim(image_dim.width, image_dim.height)

    def _shape(self):
        return (self.image_dims_.height, self.image_dims_.width)

    def InitFrame(self, color_space: COLOR_SPACE, color_image) -> None:
        rgba = _rgba(color_image, self._shape())
        check(self._lib.dtsgb_dts_init_frame(self._h, int(color_space),
                                             _ptr(rgba), None, None))

    def Filter(self, filter_params: DomainFilterParams, input_, num_iter: int = 3):
        inp = _f32(input_, self._shape())
        out = np.empty(self._shape(), np.float32)
        check(self._lib.dtsgb_dts_filter(self._h, ctypes.byref(filter_params._c()),
                                         _ptr(inp), _ptr(out), int(num_iter)))
        return out

    def Download(self, image_type: ImageType) -> np.ndarray:
        h, w = self._shape()
        if int(image_type) == ImageType.COLOR_IMAGE:
            out = np.zeros((h, w, 4), np.uint8)
        else:
            out = np.zeros((h, w), np.float32)
        check(self._lib.dtsgb_dts_download(self._h, int(image_type), _ptr(out)))
        return out

    def ClearAll(self) -> None:
        check(self._lib.dtsgb_dts_clear_all(self._h))

    def ComputeColorSpaceDifferential(self, params: DomainFilterParams) -> None:
        check(self._lib.dtsgb_dts_compute_differential(self._h, ctypes.byref(params._c())))

    def IntegrateColorDifferentials(self) -> None:
        check(self._lib.dtsgb_dts_integrate(self._h))

    def DebugBounds(self, axis: int, sigma: float):
        """Window bounds (l, u] the kernels use for one sigma (tests)."""
        h, w = self._shape()
        l = np.empty((h, w), np.int32)
        u = np.empty((h, w), np.int32)
        check(self._lib.dtsgb_dts_debug_bounds(self._h, int(axis), float(sigma),
                                               _ptr(l), _ptr(u)))
        return l, u


class DomainTransformSolver(DomainTransformFilter):
    """src/domain_transform_solver.h:34-85."""

    _flags_base = 0

    def InitFrame(self, color_space: COLOR_SPACE, color_image, target=None,
                  confidence=None) -> None:
        shape = self._shape()
        rgba = _rgba(color_image, shape)
        t = _f32(target, shape) if target is not None else None
        c = _f32(confidence, shape) if confidence is not None else None
        check(self._lib.dtsgb_dts_init_frame(self._h, int(color_space), _ptr(rgba),
                                             _ptr(t), _ptr(c)))

    def UploadTargets(self, target, confidence=None) -> None:
        """New target and confidence for the guide in place (video frames
        with a fixed guide); the next Optimize with the same sigma_z keeps
        the window bounds (dtsgb_dts_upload_targets)."""
        shape = self._shape()
        t = _f32(target, shape)
        c = _f32(confidence, shape) if confidence is not None else None
        check(self._lib.dtsgb_dts_upload_targets(self._h, _ptr(t), _ptr(c)))

    def Optimize(self, optimize_params: DomainOptimizeParams,
                 overwrite_target_above_conf: float = -1) -> None:
        check(self._lib.dtsgb_dts_optimize(self._h, ctypes.byref(optimize_params._c()),
                                           float(overwrite_target_above_conf)))

    def ComputeConfidence(self, conf_params: DomainFilterParamsVec1,
                          left_side_clear_width: int) -> None:
        check(self._lib.dtsgb_dts_compute_confidence(
            self._h, ctypes.byref(conf_params._c()), int(left_side_clear_width)))


class DomainTransformStereo(DomainTransformSolver):
    """src/domain_transform_stereo.h:93-114: the solver plus a right image;
    Optimize adds the photometric term of PhotometricL2LossTerm."""

    _flags_base = FLAG_STEREO

    def InitRightFrame(self, center_offset: float, color_space: COLOR_SPACE,
                       color_image) -> None:
        rgba = _rgba(color_image, self._shape())
        check(self._lib.dtsgb_dts_init_right_frame(self._h, float(center_offset),
                                                   int(color_space), _ptr(rgba)))

    def ProcessRightFrame(self) -> None:
        check(self._lib.dtsgb_dts_process_right_frame(self._h))


class HFBS:
    """src/hfbs.h:99-150."""

    def __init__(self, max_image_dims: ImageDim, max_grid_x: int,
                 max_grid_y: int, max_grid_l: int, flags: int = 0):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.dtsgb_hfbs_create(max_image_dims.width,
                                          max_image_dims.height, max_grid_x,
                                          max_grid_y, max_grid_l, flags,
                                          ctypes.byref(h)))
        self._h = h
        self.image_dim_ = ImageDim(max_image_dims.width, max_image_dims.height)
        self.grid_params_ = HFBSGridParams()

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dtsgb_hfbs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def SetStream(self, stream_handle: int | None) -> None:
        check(self._lib.dtsgb_hfbs_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def _shape(self):
        return (self.image_dim_.height, self.image_dim_.width)

    def SetImageDim(self, image_dim: ImageDim) -> None:
        check(self._lib.dtsgb_hfbs_set_image_dim(self._h, image_dim.width,
                                                 image_dim.height))
        self.image_dim_ = ImageDim(image_dim.width, image_dim.height)

    def InitFrame(self, color_space: COLOR_SPACE, color_image, target,
                  confidence=None) -> None:
        shape = self._shape()
        rgba = _rgba(color_image, shape)
        t = _f32(target, shape)
        c = _f32(confidence, shape) if confidence is not None else None
        check(self._lib.dtsgb_hfbs_init_frame(self._h, int(color_space), _ptr(rgba),
                                              _ptr(t), _ptr(c)))

    def UploadTargets(self, target, confidence=None) -> None:
        """New target and confidence for the guide in place; the next
        Optimize with the same grid parameters keeps the bistochastized
        normalisation (dtsgb_hfbs_upload_targets)."""
        shape = self._shape()
        t = _f32(target, shape)
        c = _f32(confidence, shape) if confidence is not None else None
        check(self._lib.dtsgb_hfbs_upload_targets(self._h, _ptr(t), _ptr(c)))

    def SetFilterParams(self, grid_params: HFBSGridParams) -> None:
        self.grid_params_ = grid_params
        check(self._lib.dtsgb_hfbs_set_filter_params(self._h,
                                                     ctypes.byref(grid_params._c())))

    def ClearAll(self) -> None:
        check(self._lib.dtsgb_hfbs_clear_all(self._h))

    def Optimize(self) -> None:
        st = check(self._lib.dtsgb_hfbs_optimize(self._h), allow_warning=True)
        if st == _lib.DTSGB_WARN_GRID_TOO_LARGE:
            warnings.warn(self._lib.dtsgb_last_error().decode())

    def InitFrameDevice(self, color_space: COLOR_SPACE, rgba_ptr: int, target_ptr: int,
                        confidence_ptr: int | None = None) -> None:
        """InitFrame from device buffers (W*H uchar4 / float32), enqueued on
        the handle's stream."""
        check(self._lib.dtsgb_hfbs_init_frame_device(
            self._h, int(color_space), ctypes.c_void_p(rgba_ptr), ctypes.c_void_p(target_ptr),
            ctypes.c_void_p(confidence_ptr) if confidence_ptr else None))

    def DownloadDevice(self, image_type: ImageType, dst_ptr: int) -> None:
        check(self._lib.dtsgb_hfbs_download_device(self._h, int(image_type),
                                                   ctypes.c_void_p(dst_ptr)))

    def GridDims(self):
        gx, gy, gl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self._lib.dtsgb_hfbs_grid_dims(self._h, ctypes.byref(gx),
                                             ctypes.byref(gy), ctypes.byref(gl)))
        return gx.value, gy.value, gl.value

    def DebugGrid(self, which: int) -> np.ndarray:
        gx, gy, gl = self.GridDims()
        out = np.empty((gl, gy, gx), np.float32)
        check(self._lib.dtsgb_hfbs_debug_grid(self._h, int(which), _ptr(out)))
        return out

    def Download(self, image_type: ImageType) -> np.ndarray:
        out = np.zeros(self._shape(), np.float32)
        check(self._lib.dtsgb_hfbs_download(self._h, int(image_type), _ptr(out)))
        return out

    # ---- gradients (an addition; the reference has none) ------------------
    def EnableGrad(self, enable: bool = True, segment: int = 0) -> None:
        """Keep what the adjoint needs in the following Optimize calls
        (segment 0: automatic checkpoint choice)."""
        check(self._lib.dtsgb_hfbs_enable_grad(self._h, int(bool(enable)), int(segment)))

    def GradInfo(self):
        """(checkpoint segment, grid planes) of the last Optimize."""
        seg, planes = ctypes.c_int(), ctypes.c_int()
        check(self._lib.dtsgb_hfbs_grad_info(self._h, ctypes.byref(seg),
                                             ctypes.byref(planes)))
        return seg.value, planes.value

    def Backward(self, grad_out):
        """dL/dtarget, dL/dconfidence of the last Optimize for dL/doutput."""
        shape = self._shape()
        g = _f32(grad_out, shape)
        gt = np.empty(shape, np.float32)
        gc = np.empty(shape, np.float32)
        check(self._lib.dtsgb_hfbs_backward(self._h, _ptr(g), _ptr(gt), _ptr(gc)))
        return gt, gc

    def BackwardDevice(self, grad_out_ptr: int, grad_target_ptr: int | None,
                       grad_confidence_ptr: int | None) -> None:
        """Device-pointer backward (W*H float32 planes, enqueued on the
        handle's stream)."""
        check(self._lib.dtsgb_hfbs_backward_device(
            self._h, ctypes.c_void_p(grad_out_ptr),
            ctypes.c_void_p(grad_target_ptr) if grad_target_ptr else None,
            ctypes.c_void_p(grad_confidence_ptr) if grad_confidence_ptr else None))


def _ptr_array(arrays):
    n = len(arrays)
    out = (ctypes.c_void_p * n)()
    for i, a in enumerate(arrays):
        out[i] = None if a is None else a.ctypes.data
    return out


def _vp_array(ptrs):
    """ctypes array of device addresses (ints; None or 0 = skip)."""
    n = len(ptrs)
    out = (ctypes.c_void_p * n)()
    for i, p in enumerate(ptrs):
        out[i] = None if not p else int(p)
    return out


class Batch:
    """Many images of uneven size solved together (no reference counterpart:
    the reference solves one image per object).  solve_dts / solve_hfbs run
    the per-image semantics of DomainTransformSolver / HFBS on every
    instance with single launches; the launch sequence is replayed from a
    CUDA graph while the parameters stay the same."""

    def __init__(self, sizes, flags: int = 0, use_graphs: bool = True):
        self._lib = _lib.load()
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        n = len(self.sizes)
        ws = (ctypes.c_int * n)(*[w for w, _ in self.sizes])
        hs = (ctypes.c_int * n)(*[h for _, h in self.sizes])
        b = ctypes.c_void_p()
        check(self._lib.dtsgb_batch_create(n, ws, hs, flags, ctypes.byref(b)))
        self._h = b
        check(self._lib.dtsgb_batch_use_graphs(b, int(use_graphs)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dtsgb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle: int | None) -> None:
        check(self._lib.dtsgb_batch_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def upload(self, color_space: COLOR_SPACE, rgba, target, confidence=None) -> None:
        rg = [_rgba(a, (h, w)) for a, (w, h) in zip(rgba, self.sizes)]
        tg = [_f32(a, (h, w)) for a, (w, h) in zip(target, self.sizes)]
        cf = None
        if confidence is not None:
            cf = [None if a is None else _f32(a, (h, w))
                  for a, (w, h) in zip(confidence, self.sizes)]
        self._keep = (rg, tg, cf)
        check(self._lib.dtsgb_batch_upload(self._h, int(color_space), _ptr_array(rg),
                                           _ptr_array(tg),
                                           None if cf is None else _ptr_array(cf)))

    def upload_targets(self, target, confidence=None) -> None:
        """New target / confidence for the same guides (video frames): the
        guide-derived window bounds and HFBS normalisation are kept."""
        tg = [_f32(a, (h, w)) for a, (w, h) in zip(target, self.sizes)]
        cf = None
        if confidence is not None:
            cf = [None if a is None else _f32(a, (h, w))
                  for a, (w, h) in zip(confidence, self.sizes)]
        self._keep_t = (tg, cf)
        check(self._lib.dtsgb_batch_upload_targets(self._h, _ptr_array(tg),
                                                   None if cf is None else _ptr_array(cf)))

    def solve_dts(self, filter_params: DomainFilterParams,
                  optimize_params: DomainOptimizeParams,
                  overwrite_target_above_conf: float = -1) -> None:
        check(self._lib.dtsgb_batch_solve_dts(self._h, ctypes.byref(filter_params._c()),
                                              ctypes.byref(optimize_params._c()),
                                              float(overwrite_target_above_conf)))

    def solve_hfbs(self, grid_params: HFBSGridParams) -> None:
        check(self._lib.dtsgb_batch_solve_hfbs(self._h, ctypes.byref(grid_params._c())))

    def download(self, which: int):
        """which: 0 = DTS result, 1 = HFBS result."""
        outs = [np.empty((h, w), np.float32) for w, h in self.sizes]
        check(self._lib.dtsgb_batch_download(self._h, int(which), _ptr_array(outs)))
        return outs

    def debug_bounds(self, i: int):
        """Windows of instance i's last DTS solve as absolute indices along
        each axis: (l_x, u_x, l_y, u_y), the window being (l, u]."""
        w, h = self.sizes[i]
        packed = np.empty((h, w), np.uint32)
        check(self._lib.dtsgb_batch_debug_plane(self._h, int(i), 0, _ptr(packed),
                                                packed.nbytes))
        xs = np.arange(w, dtype=np.int32)[None, :]
        ys = np.arange(h, dtype=np.int32)[:, None]
        b = packed.astype(np.int64)
        return (xs - (b & 0xFF)).astype(np.int32), (xs + ((b >> 8) & 0xFF)).astype(np.int32), \
            (ys - ((b >> 16) & 0xFF)).astype(np.int32), (ys + (b >> 24)).astype(np.int32)

    def debug_grid(self, i: int, which: int, grid_dims):
        """HFBS grid of instance i's last solve, shape (gl, gy, gx): which 1 =
        splat counts, 2 = splatted confidences, 3 = splatted c * t."""
        gx, gy, gl = grid_dims
        out = np.empty((gl, gy, gx), np.float32)
        check(self._lib.dtsgb_batch_debug_plane(self._h, int(i), int(which), _ptr(out),
                                                out.nbytes))
        return out

    # ---- device pointers (integers), e.g. from torch tensors ----------------
    def upload_device(self, color_space: COLOR_SPACE, rgba_ptrs, target_ptrs,
                      confidence_ptrs=None) -> None:
        conf = None if confidence_ptrs is None else _vp_array(confidence_ptrs)
        check(self._lib.dtsgb_batch_upload_device(self._h, int(color_space),
                                                  _vp_array(rgba_ptrs),
                                                  _vp_array(target_ptrs), conf))

    def download_device(self, which: int, dst_ptrs) -> None:
        check(self._lib.dtsgb_batch_download_device(self._h, int(which),
                                                    _vp_array(dst_ptrs)))

    # ---- tuning (no reference counterpart) ----------------------------------
    def set_tuning(self, knob: int, value: int) -> None:
        check(self._lib.dtsgb_batch_set_tuning(self._h, int(knob), int(value)))

    def get_tuning(self, knob: int) -> int:
        v = ctypes.c_longlong()
        check(self._lib.dtsgb_batch_get_tuning(self._h, int(knob), ctypes.byref(v)))
        return v.value

    def tuning(self) -> dict:
        """Every knob's current value, by name."""
        return {name: self.get_tuning(k) for k, name in TUNE_NAMES.items()}

    def autotune(self, filter_params=None, optimize_params=None, grid_params=None,
                 overwrite_target_above_conf: float = -1, reps: int = 3,
                 cache_path: str | None = None) -> bool:
        """Time each tile shape, bounds segment and HFBS steps / group budget
        on the uploaded batch and keep the fastest.  With cache_path, a case
        tuned before (same device, sizes and parameters) is read from that
        file instead; returns True when it was."""
        f = None if filter_params is None else ctypes.byref(filter_params._c())
        o = None if optimize_params is None else ctypes.byref(optimize_params._c())
        g = None if grid_params is None else ctypes.byref(grid_params._c())
        if cache_path is None:
            check(self._lib.dtsgb_batch_autotune(self._h, f, o,
                                                 float(overwrite_target_above_conf), g,
                                                 int(reps)))
            return False
        hit = ctypes.c_int()
        check(self._lib.dtsgb_batch_autotune_cached(
            self._h, f, o, float(overwrite_target_above_conf), g, int(reps),
            str(cache_path).encode(), ctypes.byref(hit)))
        return bool(hit.value)

    # ---- gradients of the DTS solve (no reference counterpart) --------------
    def enable_grad(self, enable: bool = True, segment: int = 0) -> None:
        """Keep checkpoints in solve_dts every `segment` iterations
        (0 = automatic, near sqrt(N)) so that backward() can run."""
        check(self._lib.dtsgb_batch_enable_grad(self._h, int(enable), int(segment)))

    def grad_info(self):
        """(segment length, planes held) of the last solve."""
        seg, planes = ctypes.c_int(), ctypes.c_int()
        check(self._lib.dtsgb_batch_grad_info(self._h, ctypes.byref(seg),
                                              ctypes.byref(planes)))
        return seg.value, planes.value

    def backward(self, grad_out):
        """dL/dtarget, dL/dconfidence (lists of HxW float32) for the upstream
        gradients dL/dv of the last solve_dts results."""
        go = [_f32(a, (h, w)) for a, (w, h) in zip(grad_out, self.sizes)]
        gt = [np.empty((h, w), np.float32) for w, h in self.sizes]
        gc = [np.empty((h, w), np.float32) for w, h in self.sizes]
        check(self._lib.dtsgb_batch_dts_backward(self._h, _ptr_array(go), _ptr_array(gt),
                                                 _ptr_array(gc)))
        return gt, gc

    def backward_device(self, grad_out_ptrs, grad_target_ptrs, grad_conf_ptrs=None) -> None:
        gc = None if grad_conf_ptrs is None else _vp_array(grad_conf_ptrs)
        check(self._lib.dtsgb_batch_dts_backward_device(self._h, _vp_array(grad_out_ptrs),
                                                        _vp_array(grad_target_ptrs), gc))

    def hfbs_grad_info(self):
        """(segment length, grid planes) of the last differentiable
        solve_hfbs ((0, 0): none)."""
        seg, planes = ctypes.c_int(), ctypes.c_int()
        check(self._lib.dtsgb_batch_hfbs_grad_info(self._h, ctypes.byref(seg),
                                                   ctypes.byref(planes)))
        return seg.value, planes.value

    def hfbs_backward(self, grad_out):
        """dL/dtarget, dL/dconfidence (lists of HxW float32) for the upstream
        gradients of the last solve_hfbs results."""
        go = [_f32(a, (h, w)) for a, (w, h) in zip(grad_out, self.sizes)]
        gt = [np.empty((h, w), np.float32) for w, h in self.sizes]
        gc = [np.empty((h, w), np.float32) for w, h in self.sizes]
        check(self._lib.dtsgb_batch_hfbs_backward(self._h, _ptr_array(go), _ptr_array(gt),
                                                  _ptr_array(gc)))
        return gt, gc

    def hfbs_backward_device(self, grad_out_ptrs, grad_target_ptrs,
                             grad_conf_ptrs=None) -> None:
        gc = None if grad_conf_ptrs is None else _vp_array(grad_conf_ptrs)
        check(self._lib.dtsgb_batch_hfbs_backward_device(
            self._h, _vp_array(grad_out_ptrs), _vp_array(grad_target_ptrs), gc))


class Pipeline:
    """Host-to-host solves of many images with the copies of one chunk of
    instances overlapping the solves of another (dtsgb_pipeline_*): each
    chunk is a Batch-like set of consecutive instances on its own stream.
    Copies overlap only from pinned host memory (e.g. torch's
    pin_memory()); numpy arrays work but copy synchronously."""

    def __init__(self, sizes, flags: int = 0, n_chunks: int = 4):
        self._lib = _lib.load()
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        n = len(self.sizes)
        ws = (ctypes.c_int * n)(*[w for w, _ in self.sizes])
        hs = (ctypes.c_int * n)(*[h for _, h in self.sizes])
        p = ctypes.c_void_p()
        check(self._lib.dtsgb_pipeline_create(n, ws, hs, flags, int(n_chunks),
                                              ctypes.byref(p)))
        self._h = p

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dtsgb_pipeline_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def n_chunks(self) -> int:
        return int(self._lib.dtsgb_pipeline_chunks(self._h))

    def set_tuning(self, knob: int, value: int) -> None:
        """Apply a batch tuning knob (TUNE_*) to every chunk."""
        for k in range(self.n_chunks):
            b = ctypes.c_void_p()
            check(self._lib.dtsgb_pipeline_batch(self._h, k, ctypes.byref(b)))
            check(self._lib.dtsgb_batch_set_tuning(b, int(knob), int(value)))

    def run_ptrs(self, color_space: COLOR_SPACE, rgba_ptrs, target_ptrs, confidence_ptrs,
                 filter_params: DomainFilterParams | None,
                 optimize_params: DomainOptimizeParams | None,
                 grid_params: HFBSGridParams | None, out_dts_ptrs, out_hfbs_ptrs,
                 overwrite_target_above_conf: float = -1) -> None:
        """The same on raw host pointers (integers), e.g. pinned buffers."""
        dts = filter_params is not None and optimize_params is not None
        check(self._lib.dtsgb_pipeline_run(
            self._h, int(color_space), _vp_array(rgba_ptrs), _vp_array(target_ptrs),
            None if confidence_ptrs is None else _vp_array(confidence_ptrs),
            ctypes.byref(filter_params._c()) if dts else None,
            ctypes.byref(optimize_params._c()) if dts else None,
            float(overwrite_target_above_conf),
            ctypes.byref(grid_params._c()) if grid_params is not None else None,
            _vp_array(out_dts_ptrs) if dts else None,
            _vp_array(out_hfbs_ptrs) if grid_params is not None else None))

    def run(self, color_space: COLOR_SPACE, rgba, target, confidence=None,
            filter_params: DomainFilterParams | None = None,
            optimize_params: DomainOptimizeParams | None = None,
            grid_params: HFBSGridParams | None = None, overwrite_target_above_conf=-1):
        """Upload, DTS (given filter and optimize params) and HFBS (given grid
        params), download.  Returns (dts results or None, hfbs results or
        None), lists of HxW float32."""
        rg = [_rgba(a, (h, w)) for a, (w, h) in zip(rgba, self.sizes)]
        tg = [_f32(a, (h, w)) for a, (w, h) in zip(target, self.sizes)]
        cf = None
        if confidence is not None:
            cf = [None if a is None else _f32(a, (h, w))
                  for a, (w, h) in zip(confidence, self.sizes)]
        dts = filter_params is not None and optimize_params is not None
        od = [np.empty((h, w), np.float32) for w, h in self.sizes] if dts else None
        oh = ([np.empty((h, w), np.float32) for w, h in self.sizes]
              if grid_params is not None else None)
        check(self._lib.dtsgb_pipeline_run(
            self._h, int(color_space), _ptr_array(rg), _ptr_array(tg),
            None if cf is None else _ptr_array(cf),
            ctypes.byref(filter_params._c()) if dts else None,
            ctypes.byref(optimize_params._c()) if dts else None,
            float(overwrite_target_above_conf),
            ctypes.byref(grid_params._c()) if grid_params is not None else None,
            _ptr_array(od) if dts else None, _ptr_array(oh) if oh is not None else None))
        return od, oh

    def run_grad(self, color_space: COLOR_SPACE, rgba, target, confidence,
                 filter_params: DomainFilterParams, optimize_params: DomainOptimizeParams,
                 grad_out):
        """Differentiable solve: returns (v, dL/dtarget, dL/dconfidence), lists
        of HxW float32, for the upstream gradients grad_out = dL/dv."""
        rg = [_rgba(a, (h, w)) for a, (w, h) in zip(rgba, self.sizes)]
        tg = [_f32(a, (h, w)) for a, (w, h) in zip(target, self.sizes)]
        cf = None
        if confidence is not None:
            cf = [None if a is None else _f32(a, (h, w))
                  for a, (w, h) in zip(confidence, self.sizes)]
        go = [_f32(a, (h, w)) for a, (w, h) in zip(grad_out, self.sizes)]
        v = [np.empty((h, w), np.float32) for w, h in self.sizes]
        gt = [np.empty((h, w), np.float32) for w, h in self.sizes]
        gc = [np.empty((h, w), np.float32) for w, h in self.sizes]
        check(self._lib.dtsgb_pipeline_run_grad(
            self._h, int(color_space), _ptr_array(rg), _ptr_array(tg),
            None if cf is None else _ptr_array(cf), ctypes.byref(filter_params._c()),
            ctypes.byref(optimize_params._c()), _ptr_array(go), _ptr_array(v),
            _ptr_array(gt), _ptr_array(gc)))
        return v, gt, gc

# ---- generic solve API, src/edge_aware_solver.h:13-90 (cv::Mat-free) -------
@dataclass
class DtsOptions:
    filter_options: DomainFilterParams = field(default_factory=DomainFilterParams)
    optim_options: DomainOptimizeParams = field(default_factory=DomainOptimizeParams)
    conf_params: DomainFilterParamsVec1 = field(default_factory=DomainFilterParamsVec1)
    color_space: COLOR_SPACE = COLOR_SPACE.YCbCr
    image_dims: ImageDim = field(default_factory=ImageDim)
    overwrite_target_above_conf: float = -1


@dataclass
class HfbsOptions:
    grid_params: HFBSGridParams = field(default_factory=HFBSGridParams)
    color_space: COLOR_SPACE = COLOR_SPACE.YCbCr
    image_dims: ImageDim = field(default_factory=ImageDim)
    overwrite_target_above_conf: float = -1


def Solve(options, compute_confidence: bool, solver) -> None:
    """Solve<DtsOptions> / Solve<HfbsOptions>, edge_aware_solver.h:37-55."""
    if isinstance(options, DtsOptions):
        solver.ComputeColorSpaceDifferential(options.filter_options)
        solver.IntegrateColorDifferentials()
        if compute_confidence:
            solver.ComputeConfidence(options.conf_params, 0)
        solver.Optimize(options.optim_options, options.overwrite_target_above_conf)
    elif isinstance(options, HfbsOptions):
        solver.Optimize()
    else:
        raise TypeError("options must be DtsOptions or HfbsOptions")


def EdgeAwareOptimize(rgba_image, target_image, confidence, options, solver):
    """EdgeAwareOptimize, edge_aware_solver.h:59-90, without OpenCV: returns
    (solution, host wall time in ms of Solve plus the blocking Download).
    bench.py times the solve alone with CUDA events."""
    import time

    solver.SetImageDim(options.image_dims)
    solver.ClearAll()
    if isinstance(solver, HFBS):
        solver.SetFilterParams(options.grid_params)
    solver.InitFrame(options.color_space, rgba_image, target_image, confidence)
    t0 = time.perf_counter()
    Solve(options, confidence is None, solver)
    out = solver.Download(ImageType.OPTIMIZED_QUANTITY)
    return out, (time.perf_counter() - t0) * 1e3


class SoftDTS:
    """Soft-window DTS over device buffers (no reference counterpart): the
    Optimize iteration with fractional window ends of width tau, so that the
    result is differentiable in the edge weights dH, dV (the reference's
    integer windows make that gradient zero almost everywhere).  Arguments
    are lists of device pointers (ints), one per instance, as in
    include/dtsgb.h's dtsgb_soft_* calls."""

    def __init__(self, sizes):
        self._lib = _lib.load()
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        n = len(self.sizes)
        ws = (ctypes.c_int * n)(*[w for w, _ in self.sizes])
        hs = (ctypes.c_int * n)(*[h for _, h in self.sizes])
        s = ctypes.c_void_p()
        check(self._lib.dtsgb_soft_create(n, ws, hs, ctypes.byref(s)))
        self._h = s

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.dtsgb_soft_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None) -> None:
        check(self._lib.dtsgb_soft_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def edge_weights(self, color_space, rgba_ptrs, filter_params, dh_ptrs, dv_ptrs) -> None:
        check(self._lib.dtsgb_soft_edge_weights(self._h, int(color_space),
                                                _vp_array(rgba_ptrs),
                                                ctypes.byref(filter_params._c()),
                                                _vp_array(dh_ptrs), _vp_array(dv_ptrs)))

    def solve(self, dh_ptrs, dv_ptrs, target_ptrs, confidence_ptrs, optimize_params,
              tau: float, out_ptrs) -> None:
        conf = None if confidence_ptrs is None else _vp_array(confidence_ptrs)
        check(self._lib.dtsgb_soft_solve(self._h, _vp_array(dh_ptrs), _vp_array(dv_ptrs),
                                         _vp_array(target_ptrs), conf,
                                         ctypes.byref(optimize_params._c()), float(tau),
                                         _vp_array(out_ptrs)))

    def backward(self, grad_out_ptrs, grad_t_ptrs=None, grad_c_ptrs=None, grad_dh_ptrs=None,
                 grad_dv_ptrs=None) -> None:
        def arr(p):
            return None if p is None else _vp_array(p)
        check(self._lib.dtsgb_soft_backward(self._h, _vp_array(grad_out_ptrs),
                                            arr(grad_t_ptrs), arr(grad_c_ptrs),
                                            arr(grad_dh_ptrs), arr(grad_dv_ptrs)))
