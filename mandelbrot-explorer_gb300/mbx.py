"""Host-side mirror of the reference's compute-backend plugin API over the C ABI.

The reference selects a renderer with ``createComputeBackend(name)`` and calls
``IComputeBackend::compute(const ComputeRequest&)`` (cbotx/Mandelbrot-Explorer
src/engine/compute_backend.h:17-117). This module exposes the same names and
argument meanings for the "cuda" backend implemented by
``lib/libmbx_gb300.so`` (declared in ``include/mbx_gb300.h``):

    backend = create_compute_backend("cuda")
    req = ComputeRequest(center_re="-0.75", center_im="0.1", scale="2" + "0"*30,
                         width=1280, height=720, max_iterations=50000)
    ok = backend.compute(req)          # fills req.iterations (numpy float32)

There is no CPU fallback: when the library or a CUDA device is unavailable,
``create_compute_backend`` raises.
"""
from __future__ import annotations

import ctypes
import math
import os
import threading
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmbx_gb300.so")

# ColoringMethod bits (src/engine/mandel_perturbation.h:30-49).
SUPER_SAMPLING = 1
EXTERIOR_DIST_EST = 2
NORMAL_MAP = 16
DE_OVERLAY = 64
MODE_MANDELBROT, MODE_JULIA = 0, 1
EMPTYPIXEL = -10.0

PRECISION_EXACT = 0
PRECISION_MIXED = 1

OK, E_INVALID, E_CUDA, E_CANCELLED, E_NODEVICE, E_BUSY, E_NOMEM, E_TOO_LARGE = 0, -1, -2, -3, -4, -5, -6, -7


class _Request(ctypes.Structure):
    _fields_ = [
        ("center_re", ctypes.c_char_p),
        ("center_im", ctypes.c_char_p),
        ("scale", ctypes.c_char_p),
        ("precision_bits", ctypes.c_int),
        ("width", ctypes.c_int),
        ("height", ctypes.c_int),
        ("full_height", ctypes.c_int),
        ("row_base", ctypes.c_int),
        ("sub", ctypes.c_int),
        ("max_iterations", ctypes.c_int),
        ("coloring_method", ctypes.c_int),
        ("bailout", ctypes.c_double),
        ("precision_mode", ctypes.c_int),
        ("outputs_on_device", ctypes.c_int),
        ("iterations", ctypes.c_void_p),
        ("normal", ctypes.c_void_p),
        ("escape_iteration", ctypes.c_void_p),
        ("progress", ctypes.c_void_p),
        ("reuse_reference", ctypes.c_int),
        ("compute_mode", ctypes.c_int),
        ("fixed_c_re", ctypes.c_char_p),
        ("fixed_c_im", ctypes.c_char_p),
        ("reference_re", ctypes.c_char_p),
        ("reference_im", ctypes.c_char_p),
        ("reference_period", ctypes.c_int),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [
        ("threads", ctypes.c_int),
        ("blocks_per_sm", ctypes.c_int),
        ("smem_orbit_limit", ctypes.c_int),
        ("rescale_window", ctypes.c_double),
        ("pass_ms", ctypes.c_double),
        ("lane_budget", ctypes.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(ctypes.Structure):
    _fields_ = [
        ("total_ms", ctypes.c_double),
        ("orbit_ms", ctypes.c_double),
        ("bla_ms", ctypes.c_double),
        ("kernel_ms", ctypes.c_double),
        ("copy_ms", ctypes.c_double),
        ("steps", ctypes.c_longlong),
        ("bla_applies", ctypes.c_longlong),
        ("bla_skipped", ctypes.c_longlong),
        ("effective_iterations", ctypes.c_longlong),
        ("gmp_pixels", ctypes.c_longlong),
        ("samples", ctypes.c_longlong),
        ("passes", ctypes.c_int),
        ("references", ctypes.c_int),
        ("method", ctypes.c_int),
        ("used_floatexp", ctypes.c_int),
        ("period", ctypes.c_int),
        ("reference_length", ctypes.c_int),
        ("kernel_launches", ctypes.c_int),
        ("interior", ctypes.c_int),
        ("pass_gpu_ms", ctypes.c_double),
        ("reused_reference", ctypes.c_int),
        ("rebases", ctypes.c_longlong),
        ("fp64_reruns", ctypes.c_longlong),
        ("rerun_gpu_ms", ctypes.c_double),
        ("fp64_reruns_fp64", ctypes.c_longlong),
        ("rerun_fp64_gpu_ms", ctypes.c_double),
        ("exact_steps", ctypes.c_longlong),
        ("fe_rebases", ctypes.c_longlong),
        ("exact_reruns", ctypes.c_longlong),
        ("h2d_bytes", ctypes.c_longlong),
        ("d2h_bytes", ctypes.c_longlong),
        ("fp32_pass_gpu_ms", ctypes.c_double),
        ("fp32_pass_steps", ctypes.c_longlong),
        ("fp32_pass_bla_applies", ctypes.c_longlong),
        ("fp32_unvouched_interior", ctypes.c_longlong),
        ("fp32_unvouched_escape", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every symbol declared in include/mbx_gb300.h.
EXPORTS = (
    "mbx_create",
    "mbx_destroy",
    "mbx_compute",
    "mbx_cancel",
    "mbx_reset_cancellation",
    "mbx_info_name",
    "mbx_info_detail",
    "mbx_last_error",
    "mbx_abi_version",
    "mbx_find_nucleus",
    "mbx_measure_fma_peak",
    "mbx_render_shallow_noalloc",
    "mbx_set_tuning",
    "mbx_set_lane_budget",
    "mbx_autotune",
    "mbx_compute_batch",
    "mbx_set_batch_scheduling",
    "mbx_set_batch_direct",
    "mbx_schedule_params",
    "mbx_schedule_gradient",
    "mbx_color_defaults",
    "mbx_colorize",
    "mbx_render_image",
    "mbx_last_color_stats",
    "mbx_write_bmp",
    "mbx_color_tables",
)

# Image epilogue (render.cpp colouring): value mappings and shadings.
MAP_LOG_POWER, MAP_DISTANCE, MAP_STRIPE, MAP_TRAP = 0, 1, 2, 3
SHADE_NONE, SHADE_RELIEF, SHADE_NORMAL_MAP, SHADE_DE_OVERLAY = 0, 1, 2, 3
GAMMA_STEPS = 352


class ColorParams(ctypes.Structure):
    """mbx_color_params; defaults are the render tool's (render.cpp:21, 44-46)."""

    _fields_ = [
        ("supersample", ctypes.c_int),
        ("mapping", ctypes.c_int),
        ("shading", ctypes.c_int),
        ("density", ctypes.c_float),
        ("light_az", ctypes.c_double),
        ("light_el", ctypes.c_double),
        ("relief_strength", ctypes.c_double),
        ("de_k", ctypes.c_double),
    ]

    def __init__(self, **kw):
        super().__init__(1, MAP_LOG_POWER, SHADE_NONE, 60.0, 2.3, 0.55, 1.0, 1.5)
        for k, v in kw.items():
            if k not in dict(self._fields_):
                raise TypeError("unknown colour parameter %r" % k)
            setattr(self, k, v)

SCHED_PARAMS = 64 * 24 + 64 + 64 * 64 + 64 + 64 + 1

_lib = None
_lib_lock = threading.Lock()


def load_library(path: Optional[str] = None, build_if_missing: bool = True):
    """Load libmbx_gb300.so (building it in-tree if absent); raises on failure."""
    global _lib
    with _lib_lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p) and build_if_missing:
            import importlib.util

            spec = importlib.util.spec_from_file_location("mbx_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        lib = ctypes.CDLL(p)
        lib.mbx_create.restype = ctypes.c_void_p
        lib.mbx_create.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
        lib.mbx_destroy.argtypes = [ctypes.c_void_p]
        lib.mbx_compute.restype = ctypes.c_int
        lib.mbx_compute.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Request), ctypes.POINTER(Stats)]
        lib.mbx_cancel.argtypes = [ctypes.c_void_p]
        lib.mbx_reset_cancellation.argtypes = [ctypes.c_void_p]
        for fn in ("mbx_info_name", "mbx_info_detail", "mbx_last_error"):
            getattr(lib, fn).restype = ctypes.c_char_p
            getattr(lib, fn).argtypes = [ctypes.c_void_p]
        lib.mbx_abi_version.restype = ctypes.c_int
        lib.mbx_measure_fma_peak.restype = ctypes.c_int
        lib.mbx_measure_fma_peak.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.mbx_set_tuning.restype = ctypes.c_int
        lib.mbx_set_tuning.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        lib.mbx_set_lane_budget.restype = ctypes.c_int
        lib.mbx_set_lane_budget.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.mbx_autotune.restype = ctypes.c_int
        lib.mbx_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Request), ctypes.POINTER(Tuning)]
        lib.mbx_set_batch_scheduling.restype = ctypes.c_int
        lib.mbx_set_batch_scheduling.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.mbx_set_batch_direct.restype = ctypes.c_int
        lib.mbx_set_batch_direct.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
        lib.mbx_schedule_params.restype = ctypes.c_int
        lib.mbx_schedule_params.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.mbx_schedule_gradient.restype = ctypes.c_int
        lib.mbx_schedule_gradient.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.mbx_compute_batch.restype = ctypes.c_int
        lib.mbx_compute_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Request), ctypes.c_int, ctypes.POINTER(Stats), ctypes.POINTER(Stats)]
        lib.mbx_render_shallow_noalloc.restype = ctypes.c_int
        lib.mbx_render_shallow_noalloc.argtypes = [ctypes.c_double] * 4 + [ctypes.c_int] * 3 + [ctypes.c_double, ctypes.c_int] + [ctypes.c_void_p] * 4
        lib.mbx_find_nucleus.restype = ctypes.c_int
        lib.mbx_find_nucleus.argtypes = [ctypes.c_char_p] * 3 + [ctypes.c_int] * 2 + [ctypes.c_char_p] * 2 + [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.mbx_color_defaults.argtypes = [ctypes.POINTER(ColorParams)]
        lib.mbx_colorize.restype = ctypes.c_int
        lib.mbx_colorize.argtypes = [ctypes.c_void_p, ctypes.POINTER(ColorParams), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.mbx_render_image.restype = ctypes.c_int
        lib.mbx_render_image.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Request), ctypes.POINTER(ColorParams), ctypes.c_void_p, ctypes.POINTER(Stats)]
        lib.mbx_last_color_stats.restype = ctypes.c_int
        lib.mbx_last_color_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]
        lib.mbx_write_bmp.restype = ctypes.c_int
        lib.mbx_write_bmp.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.mbx_color_tables.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        if path is None:
            _lib = lib
        return lib


def precision_for_scale(scale: str) -> int:
    """render.cpp:170-174 / verify.cpp runCase: bits = digits(scale)*log2(10)+64."""
    digits = sum(ch.isdigit() for ch in scale)
    return int(digits * math.log(10) / math.log(2)) + 64


def scale_digits(exponent: int, mantissa: str = "1") -> str:
    """Decimal digit string for mantissa * 10**exponent (the reference tools' scale form)."""
    return mantissa + "0" * exponent


@dataclass
class ComputeBackendInfo:
    """compute_backend.h:53-58."""

    name: str
    detail: str
    hardware_accelerated: bool = True
    fallback: bool = False


@dataclass
class ComputeRequest:
    """ComputeRequest (compute_backend.h:17-51), Mandelbrot mode.

    ``scale`` is the reference's mpf scale as a decimal string: the view
    half-width is 2/scale. Output buffers are allocated when left None:
    ``iterations`` (float32, reference layout), ``normal`` (DE overlay) and
    ``escape_iteration`` (int32 N per sample, -1 interior, -10 empty).
    Passing torch CUDA tensors keeps the outputs on the device.
    """

    center_re: str
    center_im: str
    scale: str
    width: int
    height: int
    max_iterations: int
    sub: int = 1
    coloring_method: int = 0
    full_height: int = 0
    row_base: int = 0
    bailout: float = 1e8
    precision_bits: int = 0
    precision_mode: int = PRECISION_EXACT
    iterations: object = None
    normal: object = None
    escape_iteration: object = None
    want_escape_iteration: bool = True
    progress: Optional[ctypes.c_float] = None
    reuse_reference: bool = False
    compute_mode: int = 0  # MODE_MANDELBROT / MODE_JULIA (ComputeMode)
    fixed_c_re: Optional[str] = None  # Julia: the fixed c
    fixed_c_im: Optional[str] = None
    reference_re: Optional[str] = None  # optional periodic reference (zoom sequences): nucleus and period
    reference_im: Optional[str] = None
    reference_period: int = 0

    def sample_count(self) -> int:
        return self.width * self.height * self.sub * self.sub


class CudaComputeBackend:
    """IComputeBackend (compute_backend.h:106-117) for the GB300 renderer."""

    def __init__(self, device: int = 0):
        self._lib = load_library()
        err = ctypes.create_string_buffer(512)
        ctx = self._lib.mbx_create(device, err, 512)
        if not ctx:
            raise RuntimeError("CUDA backend unavailable: " + err.value.decode(errors="replace"))
        self._ctx = ctypes.c_void_p(ctx)
        self.last_stats = Stats()
        self.last_status = OK

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.mbx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> ComputeBackendInfo:
        return ComputeBackendInfo(self._lib.mbx_info_name(self._ctx).decode(), self._lib.mbx_info_detail(self._ctx).decode())

    def last_compute_used_gpu_path(self) -> bool:
        return True

    def last_error(self) -> str:
        return self._lib.mbx_last_error(self._ctx).decode(errors="replace")

    def cancel(self):
        self._lib.mbx_cancel(self._ctx)

    def reset_cancellation(self):
        self._lib.mbx_reset_cancellation(self._ctx)

    @staticmethod
    def _ptr(buf):
        if buf is None:
            return None, False
        if isinstance(buf, np.ndarray):
            if not buf.flags["C_CONTIGUOUS"]:
                raise ValueError("output buffers must be contiguous")
            return buf.ctypes.data, False
        if hasattr(buf, "data_ptr") and getattr(buf, "is_cuda", False):
            return buf.data_ptr(), True
        raise TypeError("output buffers must be numpy arrays or torch CUDA tensors")

    def autotune(self, req: ComputeRequest) -> dict:
        """Times the mixed pass over launch shapes on `req` and keeps the fastest."""
        r, _keep = self._build(req)
        t = Tuning()
        rc = self._lib.mbx_autotune(self._ctx, ctypes.byref(r), ctypes.byref(t))
        if rc != OK:
            raise RuntimeError("autotune failed (%d): %s" % (rc, self.last_error()))
        return t.as_dict()

    def set_tuning(self, threads=256, blocks_per_sm=3, smem_orbit_limit=0, rescale_window=1e16):
        rc = self._lib.mbx_set_tuning(self._ctx, threads, blocks_per_sm, smem_orbit_limit, rescale_window)
        if rc != OK:
            raise RuntimeError("set_tuning failed (%d)" % rc)

    def set_lane_budget(self, iterations: int):
        """Iterations a mixed-pass lane walks per call between refills."""
        rc = self._lib.mbx_set_lane_budget(self._ctx, int(iterations))
        if rc != OK:
            raise RuntimeError("set_lane_budget failed (%d)" % rc)

    def compute_status(self, req: ComputeRequest) -> int:
        r, _keep = self._build(req)
        st = Stats()
        rc = self._lib.mbx_compute(self._ctx, ctypes.byref(r), ctypes.byref(st))
        self.last_stats = st
        self.last_status = rc
        return rc

    def _build(self, req: ComputeRequest):
        n = req.sample_count()
        if req.iterations is None:
            req.iterations = np.empty(n, np.float32)
        if req.normal is None and (req.coloring_method & (DE_OVERLAY | NORMAL_MAP)):
            req.normal = np.empty(n, np.float32)
        if req.escape_iteration is None and req.want_escape_iteration and isinstance(req.iterations, np.ndarray):
            req.escape_iteration = np.empty(n, np.int32)
        it, dev = self._ptr(req.iterations)
        nr, dev2 = self._ptr(req.normal)
        en, dev3 = self._ptr(req.escape_iteration)
        flags = {d for d, p in ((dev, it), (dev2, nr), (dev3, en)) if p is not None}
        if len(flags) > 1:
            raise ValueError("output buffers must all be host arrays or all be CUDA tensors")
        r = _Request(
            req.center_re.encode(),
            req.center_im.encode(),
            req.scale.encode(),
            req.precision_bits,
            req.width,
            req.height,
            req.full_height,
            req.row_base,
            req.sub,
            req.max_iterations,
            req.coloring_method,
            float(req.bailout),
            req.precision_mode,
            1 if dev else 0,
            it,
            nr,
            en,
            ctypes.cast(ctypes.pointer(req.progress), ctypes.c_void_p) if req.progress is not None else None,
            1 if req.reuse_reference else 0,
            req.compute_mode,
            req.fixed_c_re.encode() if req.fixed_c_re is not None else None,
            req.fixed_c_im.encode() if req.fixed_c_im is not None else None,
            req.reference_re.encode() if req.reference_re is not None else None,
            req.reference_im.encode() if req.reference_im is not None else None,
            req.reference_period,
        )
        return r, (req.iterations, req.normal, req.escape_iteration)

    def measure_fma_peak(self, fp64: bool) -> float:
        """Measured FMA issue rate of the device in TFLOP/s (FMA = 2 flops)."""
        v = ctypes.c_double(0.0)
        rc = self._lib.mbx_measure_fma_peak(self._ctx, 1 if fp64 else 0, ctypes.byref(v))
        if rc != OK:
            raise RuntimeError("peak probe failed: " + self.last_error())
        return v.value

    def compute(self, req: ComputeRequest) -> bool:
        """True on success, like IComputeBackend::compute."""
        return self.compute_status(req) == OK

    def set_batch_scheduling(self, mode: int) -> int:
        """Learned ordering of the batched main pass: 1 on, 0 off."""
        return self._lib.mbx_set_batch_scheduling(self._ctx, int(mode))

    def set_batch_direct(self, pixels: int) -> int:
        """Batch frames of at least `pixels` pixels render on their own (<= 0: never)."""
        return self._lib.mbx_set_batch_direct(self._ctx, int(pixels))

    def schedule_params(self, set_params=None) -> np.ndarray:
        """Reads (and first sets, when given) the ordering model's parameters."""
        out = np.empty(SCHED_PARAMS, np.float32)
        src = None
        if set_params is not None:
            src = np.ascontiguousarray(set_params, dtype=np.float32)
            assert src.size == SCHED_PARAMS
        rc = self._lib.mbx_schedule_params(self._ctx, src.ctypes.data if src is not None else None, out.ctypes.data)
        if rc != OK:
            raise RuntimeError("schedule_params failed (%d): %s" % (rc, self.last_error()))
        return out

    def schedule_gradient(self, features, targets) -> np.ndarray:
        """Gradients of one training step of the ordering model over all rows
        of features (n x 24, n >= 128) and targets (n), without an update."""
        x = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.empty(SCHED_PARAMS, np.float32)
        rc = self._lib.mbx_schedule_gradient(self._ctx, x.ctypes.data, t.ctypes.data, int(t.size), g.ctypes.data)
        if rc != OK:
            raise RuntimeError("schedule_gradient failed (%d): %s" % (rc, self.last_error()))
        return g

    def colorize(self, values, width: int, height: int, params: "ColorParams" = None, aux=None, rgb=None):
        """mbx_colorize: values (width*ss x height*ss, numpy or CUDA tensor) -> RGB [height][width][3].
        Device tensors in give a device tensor out (nothing copied)."""
        p = params or ColorParams()
        vp, dev = self._ptr(values)
        ap, adev = self._ptr(aux)
        if aux is not None and adev != dev:
            raise ValueError("values and aux must both be host arrays or both CUDA tensors")
        if rgb is None:
            if dev:
                import torch

                rgb = torch.empty((height, width, 3), dtype=torch.uint8, device=values.device)
            else:
                rgb = np.empty((height, width, 3), np.uint8)
        op, odev = self._ptr(rgb)
        if odev != dev:
            raise ValueError("rgb must live where values live")
        rc = self._lib.mbx_colorize(self._ctx, ctypes.byref(p), vp, ap, width, height, 1 if dev else 0, op)
        if rc != OK:
            raise RuntimeError("mbx_colorize failed (%d): %s" % (rc, self.last_error()))
        return rgb

    def render_image(self, req: "ComputeRequest", params: "ColorParams" = None) -> np.ndarray:
        """mbx_render_image: compute + colour on the device; returns the RGB image (host)."""
        p = params or ColorParams()
        r, _keep = self._build(req)
        ss = p.supersample
        out = np.empty((req.height // ss, req.width // ss, 3), np.uint8)
        st = Stats()
        rc = self._lib.mbx_render_image(self._ctx, ctypes.byref(r), ctypes.byref(p), out.ctypes.data, ctypes.byref(st))
        self.last_stats = st
        if rc != OK:
            raise RuntimeError("mbx_render_image failed (%d): %s" % (rc, self.last_error()))
        return out

    def last_color_stats(self):
        """(device ms of the last colour pass, palette coordinates that took the FP64 path)."""
        ms = ctypes.c_double(0.0)
        fb = ctypes.c_longlong(0)
        self._lib.mbx_last_color_stats(self._ctx, ctypes.byref(ms), ctypes.byref(fb))
        return ms.value, fb.value

    def compute_batch(self, reqs) -> int:
        """Renders several frames with shared passes (mbx_compute_batch).
        Sets last_view_stats (one Stats per frame) and last_batch_stats."""
        built = [self._build(q) for q in reqs]
        arr = (_Request * len(built))(*[b[0] for b in built])
        vst = (Stats * len(built))()
        bst = Stats()
        rc = self._lib.mbx_compute_batch(self._ctx, arr, len(built), vst, ctypes.byref(bst))
        self.last_view_stats = list(vst)
        self.last_batch_stats = bst
        self.last_status = rc
        return rc


def write_bmp(path: str, rgb) -> None:
    """render.cpp's writeBMP for an RGB image [height][width][3] (uint8). Host only."""
    img = np.ascontiguousarray(rgb, np.uint8)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("rgb must be [height][width][3]")
    rc = load_library().mbx_write_bmp(path.encode(), img.ctypes.data, img.shape[1], img.shape[0])
    if rc != OK:
        raise OSError("mbx_write_bmp failed (%d)" % rc)


def color_tables():
    """(palette float32 [3][2048], gamma thresholds float32 [352]) as built on this host."""
    pal = np.empty((3, 2048), np.float32)
    thr = np.empty(GAMMA_STEPS, np.float32)
    load_library().mbx_color_tables(pal.ctypes.data, thr.ctypes.data)
    return pal, thr


def create_compute_backend(requested: str = "cuda", device: int = 0) -> CudaComputeBackend:
    """createComputeBackend (compute_backend.cpp:277-290) — only "cuda"/"gpu" exist here."""
    name = (requested or "cuda").lower()
    if name not in ("cuda", "gpu", "gb300", "auto"):
        raise ValueError("unknown backend %r (this library provides only the CUDA backend)" % requested)
    return CudaComputeBackend(device)


def find_nucleus(center_re: str, center_im: str, radius: str, max_period: int, precision_bits: int):
    """Host-only nucleus search: returns (period, nucleus_re, nucleus_im, log10 size) or None."""
    lib = load_library()
    # digits of the precision plus room for the leading zeros of a small component
    n = precision_bits // 3 + 64 + 8192
    a = ctypes.create_string_buffer(n)
    b = ctypes.create_string_buffer(n)
    sz = ctypes.c_double(0.0)
    p = lib.mbx_find_nucleus(center_re.encode(), center_im.encode(), radius.encode(), max_period, precision_bits, a, b, n, ctypes.byref(sz))
    if p < 0:
        raise ValueError("mbx_find_nucleus failed (%d)" % p)
    if p == 0:
        return None
    return p, a.value.decode(), b.value.decode(), sz.value


def render(center_re, center_im, scale, width, height, max_iterations, **kw):
    """One-call convenience: returns (iterations, normal, escape_iteration, stats)."""
    be = create_compute_backend("cuda", kw.pop("device", 0))
    try:
        req = ComputeRequest(center_re, center_im, scale, width, height, max_iterations, **kw)
        rc = be.compute_status(req)
        if rc != OK:
            raise RuntimeError("mbx_compute failed (%d): %s" % (rc, be.last_error()))
        return req.iterations, req.normal, req.escape_iteration, be.last_stats.as_dict()
    finally:
        be.close()
