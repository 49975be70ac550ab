"""Learned ordering of the batched main pass (mbx_set_batch_scheduling).

* gradient check: one training step's gradients from the tensor-core kernel
  against the CPU reference (tests/order_ref.py) of the same BF16 MLP;
* ordering changes no output: a batch rendered with the learned order is
  identical to the natural order;
* gain: on a batch whose expensive samples come last in the natural order (a
  1920x1080 frame at 1e-300 followed by a 16x12 frame whose samples run
  20000 iterations without BLA), the ordered shared passes are faster once the
  model has trained on one batch (measured 8-14 %, asserted 5 %): the long
  samples start first instead of forming a tail after the cheap frame has
  drained.
"""
import numpy as np
import pytest

import mbx
import views
from conftest import load_cases
from order_ref import SP, ref_gradient

pytestmark = pytest.mark.gpu


def test_gradient_matches_cpu_reference():
    be = mbx.create_compute_backend("cuda")
    rng = np.random.RandomState(7)
    for trial in range(3):
        P = (rng.standard_normal(SP) * 0.2).astype(np.float32)
        X = rng.uniform(0.0, 1.0, (256, 24)).astype(np.float32)
        T = rng.uniform(0.0, 1.0, 256).astype(np.float32)
        got = be.schedule_params(P)
        assert np.array_equal(got, P)
        g = be.schedule_gradient(X, T)
        r = ref_gradient(P, X, T)
        for a, b in ((0, 1536), (1536, 1600), (1600, 5696), (5696, 5760), (5760, 5824), (5824, 5825)):
            scale = max(float(np.abs(r[a:b]).max()), 1e-6)
            assert float(np.abs(g[a:b] - r[a:b]).max()) <= 1e-4 * scale, (trial, a, b)
        # no update happened
        assert np.array_equal(be.schedule_params(), P)
    be.close()


def _frames():
    c = load_cases()["subpixel737"]
    heavy = dict(center_re=c["center_re"], center_im=c["center_im"], scale=c["scale"], max_iterations=20000, bailout=c["bailout"])
    return [(views.deep_view(300), 1920, 1080), (heavy, 16, 12)]


def _run(be, frames):
    reqs = [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED) for v, w, h in frames]
    assert be.compute_batch(reqs) == mbx.OK, be.last_error()
    return [(r.iterations.copy(), r.escape_iteration.copy()) for r in reqs], be.last_batch_stats.as_dict()


def test_learned_order_identical_and_faster():
    be = mbx.create_compute_backend("cuda")
    frames = _frames()
    assert be.set_batch_scheduling(0) == mbx.OK
    base, _ = _run(be, frames)
    natural = min(_run(be, frames)[1]["pass_gpu_ms"] for _ in range(3))
    assert be.set_batch_scheduling(1) == mbx.OK, be.last_error()
    out, _ = _run(be, frames)  # untrained: natural order, then trains on this batch
    for (it, en), (bit, ben) in zip(out, base):
        assert np.array_equal(en, ben) and np.array_equal(it, bit)
    assert be.set_batch_scheduling(2) == mbx.OK  # order with the trained model, no further training
    times = []
    for _ in range(3):
        out, st = _run(be, frames)
        times.append(st["pass_gpu_ms"])
        for (it, en), (bit, ben) in zip(out, base):
            assert np.array_equal(en, ben) and np.array_equal(it, bit)
    ordered = min(times)
    print("\n[order] natural %.3f ms, learned order %.3f ms (%.1f%%)" % (natural, ordered, 100.0 * (1.0 - ordered / natural)))
    assert ordered < 0.95 * natural
    be.close()
