"""The allocation-free entry point, mbx_render_shallow_noalloc.

Some callers cannot allocate device memory (applications that own all device
memory up front, real-time loops that must not allocate, plugin hosts that only
lend buffers). This entry point renders a shallow frame into the caller's own
device buffers with its scratch in a fixed device array. Checked through the
C ABI against the regular entry point (mbx_compute) on the same frame, on two
calls in a row (the scratch keeps the previous call's contents). This file is
collected last so a failure here never hides the other tests' results.
"""
import ctypes
from fractions import Fraction

import numpy as np
import pytest

import mbx

pytestmark = pytest.mark.gpu


def trunc53(q: Fraction) -> float:
    """q rounded toward zero to 53 significant bits (mpf_get_d semantics)."""
    assert q > 0
    e = q.numerator.bit_length() - q.denominator.bit_length()
    if Fraction(2) ** e > q:
        e -= 1
    m = (q * Fraction(2) ** (52 - e)).__floor__()
    return float(Fraction(m) * Fraction(2) ** (e - 52))


def test_noalloc_matches_regular_entry_point():
    torch = pytest.importorskip("torch")
    # View with a geometry whose double values are exact functions of the
    # request: centre (-0.5, 0), scale 1, 128 x 65 samples: half-width 2,
    # half-height 65/64, dx = 2*(2/127) (mpf-truncated then truncated to a
    # double), dy = 2*(65/64)/64 (exact).
    W, H, mxit = 128, 65, 3000
    # plain smooth values, exterior distance, and the distance overlay (the one
    # colouring that writes the second buffer; it takes the scalar loop)
    for cm in (0, mbx.EXTERIOR_DIST_EST, mbx.DE_OVERLAY):
        overlay = bool(cm & mbx.DE_OVERLAY)
        be = mbx.create_compute_backend("cuda")
        req = mbx.ComputeRequest("-0.5", "0", "1", W, H, mxit, coloring_method=cm, bailout=1e8)
        assert be.compute_status(req) == mbx.OK, be.last_error()
        be.close()
        c0r, c0i = -2.5, -float(Fraction(65, 64))
        dx = 2.0 * trunc53(Fraction(2, 127))
        dy = float(Fraction(65, 64) / 64 * 2)
        lib = mbx.load_library()
        it = torch.empty(W * H, dtype=torch.float32, device="cuda")
        en = torch.empty(W * H, dtype=torch.int32, device="cuda")
        nr = torch.empty(W * H, dtype=torch.float32, device="cuda") if overlay else None
        for call in range(2):
            it.fill_(123.0)
            en.fill_(7)
            if nr is not None:
                nr.fill_(55.0)
            rc = lib.mbx_render_shallow_noalloc(c0r, c0i, dx, dy, W, H, mxit, 1e8, cm, ctypes.c_void_p(it.data_ptr()), ctypes.c_void_p(en.data_ptr()),
                                                ctypes.c_void_p(nr.data_ptr()) if nr is not None else None, None)
            assert rc == mbx.OK, "cm %d call %d returned %d" % (cm, call, rc)
            got_it = it.cpu().numpy()
            got_en = en.cpu().numpy()
            assert np.array_equal(got_it.view(np.uint32), req.iterations.view(np.uint32)), "cm %d call %d: values differ" % (cm, call)
            assert np.array_equal(got_en, req.escape_iteration), "cm %d call %d: escape iterations differ" % (cm, call)
            if overlay:
                got_nr = nr.cpu().numpy()
                assert np.array_equal(got_nr.view(np.uint32), req.normal.view(np.uint32)), "call %d: overlay distances differ" % call


def test_noalloc_overlay_needs_its_buffer():
    """The distance overlay goes to the normal buffer: without one the call is rejected."""
    torch = pytest.importorskip("torch")
    lib = mbx.load_library()
    it = torch.empty(16 * 16, dtype=torch.float32, device="cuda")
    rc = lib.mbx_render_shallow_noalloc(-2.5, -1.0, 0.2, 0.1, 16, 16, 100, 1e8, mbx.DE_OVERLAY, ctypes.c_void_p(it.data_ptr()), None, None, None)
    assert rc == mbx.E_INVALID


def test_noalloc_rejects_oversized_frames():
    torch = pytest.importorskip("torch")
    lib = mbx.load_library()
    it = torch.empty(16, dtype=torch.float32, device="cuda")
    rc = lib.mbx_render_shallow_noalloc(-2.5, -1.0, 0.01, 0.01, 4096, 4096, 100, 1e8, 0, ctypes.c_void_p(it.data_ptr()), None, None, None)
    assert rc == mbx.E_TOO_LARGE
