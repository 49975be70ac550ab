"""ORACLE — test infrastructure only (tests/, __graft_entry__.smoke() and the
CPU legs of bench.py). Python access to oracle/lib/libmbx_oracle.so, the CPU
restatement of the reference's perturbation path (mbx_oracle.cpp).
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def load():
    global _lib
    if _lib is None:
        import importlib.util

        spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build_oracle.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build_oracle()
        lib = ctypes.CDLL(path)
        lib.mbx_oracle_render.restype = ctypes.c_int
        lib.mbx_oracle_render.argtypes = [ctypes.c_char_p] * 3 + [ctypes.c_int] * 6 + [ctypes.c_double] + [ctypes.c_int] * 3 + [ctypes.c_void_p] * 4
        lib.mbx_oracle_truth.restype = ctypes.c_int
        lib.mbx_oracle_truth.argtypes = [ctypes.c_char_p] * 3 + [ctypes.c_int] * 7 + [ctypes.c_double] + [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.mbx_oracle_colorize.restype = ctypes.c_int
        lib.mbx_oracle_colorize.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [ctypes.c_float] + [ctypes.c_double] * 4 + [ctypes.c_void_p]
        lib.mbx_oracle_bmp.restype = ctypes.c_long
        lib.mbx_oracle_bmp.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.mbx_oracle_palette.argtypes = [ctypes.c_void_p]
        lib.mbx_oracle_gamma_value.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.mbx_oracle_julia.restype = ctypes.c_int
        lib.mbx_oracle_julia.argtypes = [ctypes.c_char_p] * 3 + [ctypes.c_int] + [ctypes.c_char_p] * 2 + [ctypes.c_int] * 4 + [ctypes.c_double] + [ctypes.c_int] * 2 + [ctypes.c_void_p] * 2
        lib.mbx_oracle_nucleus.restype = ctypes.c_int
        lib.mbx_oracle_nucleus.argtypes = [ctypes.c_char_p] * 3 + [ctypes.c_int] * 2 + [ctypes.c_char_p] * 2 + [ctypes.c_int]
        _lib = lib
    return _lib


def palette():
    """The reference's 2048-entry palette as float32 [3][2048] (render.cpp:23-29)."""
    m = np.empty((3, 2048), np.float32)
    load().mbx_oracle_palette(m.ctypes.data)
    return m


def colorize(values, width, height, ss=1, aux=None, mapping=0, shading=0, density=60.0, light_az=2.3, light_el=0.55, relief_strength=1.0, de_k=1.5):
    """render.cpp's colouring + ss x ss linear-light downsample: uint8 [height][width][3]."""
    v = np.ascontiguousarray(values, np.float32).ravel()
    if v.size != width * height * ss * ss:
        raise ValueError("values must hold (width*ss) x (height*ss) samples")
    a = None if aux is None else np.ascontiguousarray(aux, np.float32).ravel()
    out = np.empty((height, width, 3), np.uint8)
    rc = load().mbx_oracle_colorize(v.ctypes.data, None if a is None else a.ctypes.data, width, height, ss, mapping, shading, float(density), float(light_az), float(light_el), float(relief_strength), float(de_k), out.ctypes.data)
    if rc != 0:
        raise ValueError("oracle rejected the colour parameters")
    return out


def julia(center_re, center_im, scale, fixed_c_re, fixed_c_im, width, height, max_iterations, coloring_method=0, bailout=1e8, full_height=0, row_base=0, precision_bits=0):
    """Mandel::ComputeJulia restated: (iterations float32, escape index int32)."""
    it = np.empty(width * height, np.float32)
    en = np.empty(width * height, np.int32)
    prec = precision_bits or precision_for_scale(scale)
    rc = load().mbx_oracle_julia(center_re.encode(), center_im.encode(), scale.encode(), prec, fixed_c_re.encode(), fixed_c_im.encode(), width, height, max_iterations, coloring_method, float(bailout), full_height, row_base, it.ctypes.data, en.ctypes.data)
    if rc != 0:
        raise ValueError("oracle rejected the Julia request")
    return it, en


def nucleus(center_re, center_im, radius, max_period, precision_bits):
    """findNucleus on a disk (ball period + Newton + inside check, serial as
    mp.cpp:116-223): (period, re, im) with re/im as decimal.Decimal, or None."""
    from decimal import Decimal, getcontext

    getcontext().prec = max(getcontext().prec, precision_bits // 3 + 50)
    n = precision_bits + 64
    a = ctypes.create_string_buffer(n)
    b = ctypes.create_string_buffer(n)
    p = load().mbx_oracle_nucleus(center_re.encode(), center_im.encode(), radius.encode(), max_period, precision_bits, a, b, n)
    if p < 0:
        raise ValueError("bad nucleus search input")
    if p == 0:
        return None

    def dec(s):
        d, e = s.split("@")
        neg = d.startswith("-")
        v = Decimal("0." + d.lstrip("-")).scaleb(int(e))
        return -v if neg else v

    return p, dec(a.value.decode()), dec(b.value.decode())


def gamma_value(l):
    """(int)(255 powf(l, 1/2.2) + 0.5) per linear value, as render.cpp encodes a channel."""
    l = np.ascontiguousarray(l, np.float32).ravel()
    out = np.empty(l.size, np.int32)
    load().mbx_oracle_gamma_value(l.ctypes.data, l.size, out.ctypes.data)
    return out


def bmp_bytes(rgb):
    """render.cpp's 24-bit BMP file for an RGB image [height][width][3]."""
    rgb = np.ascontiguousarray(rgb, np.uint8)
    h, w = rgb.shape[:2]
    n = load().mbx_oracle_bmp(None, w, h, None)
    buf = np.empty(n, np.uint8)
    load().mbx_oracle_bmp(rgb.ctypes.data, w, h, buf.ctypes.data)
    return buf.tobytes()


def precision_for_scale(scale):
    return int(sum(ch.isdigit() for ch in scale) * math.log(10) / math.log(2)) + 64


def render(center_re, center_im, scale, width, height, max_iterations, sub=1, coloring_method=0, bailout=1e8, full_height=0, row_base=0, threads=0, precision_bits=0):
    """Returns (iterations float32, normal float32, escape iteration int32, stats dict)."""
    lib = load()
    n = width * height * sub * sub
    it = np.empty(n, np.float32)
    nr = np.empty(n, np.float32)
    en = np.empty(n, np.int32)
    st = np.zeros(8, np.int64)
    lib.mbx_oracle_reset_rand()
    prec = precision_bits or precision_for_scale(scale)
    rc = lib.mbx_oracle_render(center_re.encode(), center_im.encode(), scale.encode(), prec, width, height, max_iterations, sub, coloring_method, float(bailout), full_height, row_base, threads, it.ctypes.data, nr.ctypes.data, en.ctypes.data, st.ctypes.data)
    if rc != 0:
        raise ValueError("oracle rejected the request (%d)" % rc)
    keys = ("steps", "bla_applies", "bla_skipped", "passes", "references", "gmp_pixels", "method")
    return it, nr, en, dict(zip(keys, (int(x) for x in st)))


def truth(center_re, center_im, scale, width, height, max_iterations, keys, sub=1, coloring_method=0, bailout=1e8, full_height=0, row_base=0, threads=0, precision_bits=0, work_bits=0):
    """Arbitrary-precision brute-force value and escape iteration of the listed
    samples (keys: (n, 4) int array of row, col, subrow, subcol)."""
    lib = load()
    keys = np.ascontiguousarray(np.asarray(keys, dtype=np.int32).reshape(-1, 4))
    n = keys.shape[0]
    out = np.empty(n, np.float32)
    nout = np.empty(n, np.int32)
    prec = precision_bits or precision_for_scale(scale)
    rc = lib.mbx_oracle_truth(center_re.encode(), center_im.encode(), scale.encode(), prec, work_bits or prec, width, height, max_iterations, sub, coloring_method, float(bailout), full_height, row_base, threads, keys.ctypes.data, n, out.ctypes.data, nout.ctypes.data)
    if rc != 0:
        raise ValueError("oracle truth rejected the request")
    return out, nout
