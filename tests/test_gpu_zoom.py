"""A zoom sequence toward a nucleus rendered with one shared periodic
reference orbit (mbx_request.reference_*): the orbit is built for the first
perturbation frame and reused by the later ones; every frame agrees with the
exact form rendered the reference's way (its own nucleus search and reference
per frame) in class and escape iteration, and its exterior distances agree
with arbitrary-precision truth on a seeded subset of each frame;
and the batched path (several frames per mbx_compute_batch call) gives the
same outputs as one frame per call."""
import os

import numpy as np
import pytest

import mbx
import zoom
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

W, H = 240, 136
FRAMES = [8, 150, 300, 450, 599]  # frame 8 is the first below half-width 2e-6 (perturbation)
# |dDE| / DE against arbitrary-precision truth (tests/golden/truth_zoom.npz):
# between scales ~1e154 and 1e280 the exact form, the reference's double path,
# carries dz/dc in FP64, whose square overflows there, and returns a distance
# of 0; the mixed form carries it as a floatexp.
DE_REL_MAX = 1e-3


def test_zoom_shared_reference_matches_exact():
    be = mbx.create_compute_backend("cuda")
    try:
        mixed = zoom.render_sequence(be, FRAMES, W, H)
        for i, (k, q, st) in enumerate(mixed):
            assert st["used_floatexp"] == 1 and st["period"] == zoom.target()[2], k
            if i == 0:
                assert st["references"] == 1 and st["reused_reference"] == 0, k
            else:
                assert st["references"] == 0 and st["reused_reference"] == 1, k
        z = np.load(os.path.join(GOLDEN, "truth_zoom.npz"))
        for k, q, st in mixed:
            e = zoom.request(k, W, H, precision_mode=mbx.PRECISION_EXACT, shared_reference=False)
            assert be.compute_status(e) == mbx.OK, be.last_error()
            mn, en = q.escape_iteration, e.escape_iteration
            valid = (q.iterations > -5) & (e.iterations > -5)
            cls = int(np.sum((mn[valid] < 0) != (en[valid] < 0)))
            same = float(np.mean(mn[valid] == en[valid]))
            # distances against arbitrary-precision truth on the frame's subset
            idx, tn, tv = z["idx_%d" % k], z["N_%d" % k], z["value_%d" % k]
            ext = (tn > 0) & (mn[idx] == tn)
            rel = np.abs(q.iterations[idx][ext].astype(np.float64) - tv[ext]) / np.abs(tv[ext]).astype(np.float64)
            erel = np.abs(e.iterations[idx][ext].astype(np.float64) - tv[ext]) / np.abs(tv[ext]).astype(np.float64)
            scale, mxit = zoom.frame_params(k)
            print("\n[zoom] frame %d (scale %s, maxiter %d): N identical to the exact form %.5f, class mismatches %d; on the truth subset N identical %.3f, "
                  "|dDE|/DE max %.3g (exact form %.3g); reruns %d, %.1f ms"
                  % (k, scale[:8] + scale[scale.index("e"):], mxit, same, cls, float(np.mean(mn[idx] == tn)), rel.max(initial=0.0), erel.max(initial=0.0), st["fp64_reruns"], st["total_ms"]))
            assert cls <= max(1, mn.size // 1000), k
            assert same >= 0.999, k
            assert float(np.mean(mn[idx] == tn)) >= 0.97, k
            assert rel.max(initial=0.0) <= DE_REL_MAX, k
    finally:
        be.close()


def test_zoom_batched_matches_single_frames():
    be = mbx.create_compute_backend("cuda")
    try:
        single = zoom.render_sequence(be, FRAMES[1:], W, H)
        batched = zoom.render_sequence(be, FRAMES[1:], W, H, batch=2)
        for (k, a, _), (k2, b, _) in zip(single, batched):
            assert k == k2
            assert np.array_equal(a.escape_iteration, b.escape_iteration), k
            assert np.array_equal(a.iterations.view(np.uint32), b.iterations.view(np.uint32)), k
    finally:
        be.close()
