"""Batched rendering (mbx_compute_batch): several frames of different sizes and
depths share one probe and one main launch sequence (a CUDA graph). Every
frame must come out identical to rendering it alone with mbx_compute, and a
replay of the same batch identical to the first run."""
import numpy as np
import pytest

import mbx
import views
from conftest import load_cases

pytestmark = pytest.mark.gpu


def _req(v, w, h, mode=mbx.PRECISION_MIXED):
    return mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], bailout=v["bailout"], precision_mode=mode)


def _frames():
    c = load_cases()
    mb = c["minibrot875"]
    sp = c["subpixel737"]
    return [
        (views.deep_view(300), 240, 135),
        (views.deep_view(1000), 160, 90),
        (dict(center_re=mb["center_re"], center_im=mb["center_im"], scale=mb["scale"], max_iterations=mb["max_iterations"], bailout=mb["bailout"]), 24, 18),
        (dict(center_re=sp["center_re"], center_im=sp["center_im"], scale=sp["scale"], max_iterations=sp["max_iterations"], bailout=sp["bailout"]), 48, 36),
        (views.c1_view(), 64, 36),  # not a floatexp frame: rendered on its own inside the batch
    ]


def test_batch_matches_single_frames():
    be = mbx.create_compute_backend("cuda")
    frames = _frames()
    singles = []
    for v, w, h in frames:
        r = _req(v, w, h)
        assert be.compute_status(r) == mbx.OK, be.last_error()
        singles.append((r.iterations.copy(), r.escape_iteration.copy()))
    for rep in range(2):  # the second run replays the captured graph
        reqs = [_req(v, w, h) for v, w, h in frames]
        rc = be.compute_batch(reqs)
        assert rc == mbx.OK, be.last_error()
        bs = be.last_batch_stats.as_dict()
        assert bs["kernel_launches"] == 8 and bs["passes"] == 2  # probe, gate, main, leftover compaction (3), double-float (2)
        for (it, en), r, (v, w, h) in zip(singles, reqs, frames):
            assert np.array_equal(r.escape_iteration, en), (rep, w, h)
            assert np.array_equal(r.iterations, it), (rep, w, h)
        print("\n[batch] run %d: samples %d, fp32 reruns %d, fp64 reruns %d, shared passes %.3f ms" % (rep, bs["samples"], bs["fp64_reruns"], bs["fp64_reruns_fp64"], bs["pass_gpu_ms"]))
    be.close()


def test_batch_device_outputs_and_invalid():
    torch = pytest.importorskip("torch")
    be = mbx.create_compute_backend("cuda")
    frames = _frames()[:2]
    reqs, host = [], []
    for v, w, h in frames:
        n = w * h
        reqs.append(mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], w, h, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED,
                                       iterations=torch.empty(n, dtype=torch.float32, device="cuda"), escape_iteration=torch.empty(n, dtype=torch.int32, device="cuda")))
        r = _req(v, w, h)
        assert be.compute_status(r) == mbx.OK
        host.append(r.escape_iteration.copy())
    assert be.compute_batch(reqs) == mbx.OK, be.last_error()
    for r, en in zip(reqs, host):
        assert np.array_equal(r.escape_iteration.cpu().numpy(), en)
    bad = _req(*frames[0])
    bad.sub = 2
    assert be.compute_batch([_req(*frames[1]), bad]) == mbx.E_INVALID
    assert "request 1" in be.last_error()
    be.close()


def test_batch_exact_form_leftovers_match_single_frames():
    """The 1080p 1e-300 frame leaves a few samples that neither the FP32 nor the
    double-float estimate vouches for; the batch hands them to the frame's exact
    form after its graph, as mbx_compute does after its tiers: same samples,
    same values."""
    be = mbx.create_compute_backend("cuda")
    assert be.set_batch_direct(0) == mbx.OK  # the 1080p frame joins the shared graph
    frames = [(views.deep_view(300), 1920, 1080), (views.deep_view(1000), 160, 90)]
    singles = []
    for v, w, h in frames:
        r = _req(v, w, h)
        assert be.compute_status(r) == mbx.OK, be.last_error()
        st = be.last_stats.as_dict()
        assert st["exact_reruns"] == st["fp64_reruns_fp64"]
        singles.append((r.iterations.copy(), r.escape_iteration.copy(), st["exact_reruns"]))
    assert singles[0][2] > 0
    reqs = [_req(v, w, h) for v, w, h in frames]
    assert be.compute_batch(reqs) == mbx.OK, be.last_error()
    bs = be.last_batch_stats.as_dict()
    assert bs["exact_reruns"] == sum(s[2] for s in singles)
    for (it, en, _), r in zip(singles, reqs):
        assert np.array_equal(r.escape_iteration, en) and np.array_equal(r.iterations, it)
    print("\n[batch] exact-form leftovers: %d" % bs["exact_reruns"])
    be.close()


def test_large_frames_render_directly_and_identically():
    """Frames of 2^20 pixels or more render on their own streams as soon as
    their host work is done (overlapping the others'), the rest in the shared
    graph; outputs are those of one-frame renders."""
    frames = [(views.deep_view(300), 1280, 820), (views.minibrot_view(), 1024, 1024), (views.deep_view(1000), 160, 90)]
    be = mbx.create_compute_backend("cuda")
    try:
        singles = []
        for v, w, h in frames:
            r = _req(v, w, h)
            assert be.compute_status(r) == mbx.OK, be.last_error()
            singles.append((r.iterations.copy(), r.escape_iteration.copy()))
        reqs = [_req(v, w, h) for v, w, h in frames]
        assert be.compute_batch(reqs) == mbx.OK, be.last_error()
        bs = be.last_batch_stats.as_dict()
        # only the small frame's probe and main samples went through the shared graph
        assert bs["samples"] < 2 * 160 * 90
        for (it, en), r, (v, w, h) in zip(singles, reqs, frames):
            assert np.array_equal(r.escape_iteration, en), (w, h)
            assert np.array_equal(r.iterations, it), (w, h)
    finally:
        be.close()
