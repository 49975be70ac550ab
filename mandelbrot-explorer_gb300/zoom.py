"""Zoom sequences: frames zooming geometrically toward a nucleus, rendered
with one periodic reference orbit shared by every frame.

The reference renders each frame of a zoom animation on its own (a nucleus
search and a reference orbit per frame, mp.cpp:1227-1386). Here every
perturbation frame of a sequence names the target nucleus and its period in
its request (mbx_request.reference_re/_im/_period): the context builds the
one-period orbit once and keeps it, and each frame redoes only its own parts
(the nucleus's position in the frame, the BLA table for the frame's radius).
The lanes of the mixed form rebase, so the one orbit serves every depth.

The zoom workload: 600 frames of 1920x1080 from half-width 1 to 1e-1000,
toward the period-72852 nucleus stored in views_data.json ("zoom"), maxiter
rising geometrically from 1e3 to 5e6, exterior distance estimation.
"""
from __future__ import annotations

import math
from decimal import Decimal, getcontext

import mbx
import views

ZOOM_FRAMES = 600
ZOOM_DEPTH = 1000          # last half-width 10^-ZOOM_DEPTH
ZOOM_MXIT = (1e3, 5e6)     # maxiter of the first and last frame
ZOOM_PRECISION = int(ZOOM_DEPTH * math.log2(10)) + 64 + 64


def target():
    """The zoom target: the nucleus and its period."""
    d = views.nucleus()["zoom"]
    return d["nucleus_re"], d["nucleus_im"], d["period"]


def frame_params(k: int, n: int = ZOOM_FRAMES, depth: int = ZOOM_DEPTH, mxit=ZOOM_MXIT):
    """Scale (decimal, half-width 2/scale) and maxiter of frame k of n: the
    half-width 10^(-depth k / (n - 1)), maxiter geometric from mxit[0] to mxit[1]."""
    t = k / (n - 1)
    getcontext().prec = 40
    scale = Decimal(2) * Decimal(10) ** (Decimal(depth) * Decimal(k) / Decimal(n - 1))
    maxiter = int(round(mxit[0] * (mxit[1] / mxit[0]) ** t))
    return format(scale, "E").replace("E+", "e"), maxiter


def request(k: int, width: int = 1920, height: int = 1080, n: int = ZOOM_FRAMES, coloring_method: int = mbx.EXTERIOR_DIST_EST,
            precision_mode: int = mbx.PRECISION_MIXED, shared_reference: bool = True, **kw) -> mbx.ComputeRequest:
    """The request of frame k: centred on the target nucleus, which is also the
    shared periodic reference (unless shared_reference is False: the engine
    then finds the frame's reference itself, as the reference does)."""
    re, im, period = target()
    scale, maxiter = frame_params(k, n)
    ref = dict(reference_re=re, reference_im=im, reference_period=period) if shared_reference else {}
    return mbx.ComputeRequest(re, im, scale, width, height, maxiter, coloring_method=coloring_method, bailout=256.0,
                              precision_bits=ZOOM_PRECISION, precision_mode=precision_mode, **ref, **kw)


def render_sequence(be: mbx.CudaComputeBackend, frames, width: int = 1920, height: int = 1080, n: int = ZOOM_FRAMES, batch: int = 1, **kw):
    """Render the listed frames (indices into the n-frame sequence) on one
    context, one mbx_compute per frame (batch = 1) or `batch` frames per
    mbx_compute_batch call. Returns [(k, request, stats dict)]."""
    out = []
    frames = list(frames)
    for i in range(0, len(frames), batch):
        ks = frames[i:i + batch]
        reqs = [request(k, width, height, n, **kw) for k in ks]
        if batch == 1:
            rc = be.compute_status(reqs[0])
            if rc != mbx.OK:
                raise RuntimeError("frame %d failed (%d): %s" % (ks[0], rc, be.last_error()))
            out.append((ks[0], reqs[0], be.last_stats.as_dict()))
        else:
            rc = be.compute_batch(reqs)
            if rc != mbx.OK:
                raise RuntimeError("frames %s failed (%d): %s" % (ks, rc, be.last_error()))
            for k, q, st in zip(ks, reqs, be.last_view_stats):
                out.append((k, q, st.as_dict()))
    return out
