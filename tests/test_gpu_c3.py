"""The batching workload (views.c3_views: 64 seed-drawn views of uneven size,
depth and maxiter, 3x3 adaptive supersampling on half of them), on an 8-view
sample at 1/16 of the linear sizes: one mbx_compute_batch call (the views'
probe and main passes in shared launches captured as one CUDA graph; the
supersampled views' extra passes after it) gives results bit-identical to
rendering each view alone, twice in a row (the second replays the graph)."""
import numpy as np
import pytest

import mbx
import views

pytestmark = pytest.mark.gpu


def request(v, **kw):
    return mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], v["width"], v["height"], v["max_iterations"], sub=v["sub"],
                              coloring_method=v["coloring_method"], bailout=v["bailout"], precision_bits=v["precision_bits"],
                              precision_mode=mbx.PRECISION_MIXED, **kw)


def test_c3_subset_batch_matches_single_views():
    vs = views.c3_views(size_div=16)[:8]
    assert any(v["sub"] > 1 for v in vs) and any(v["sub"] == 1 for v in vs)
    be = mbx.create_compute_backend("cuda")
    try:
        single = []
        for v in vs:
            q = request(v)
            assert be.compute_status(q) == mbx.OK, be.last_error()
            single.append(q)
        for rep in range(2):
            reqs = [request(v, reuse_reference=True) for v in vs]
            assert be.compute_batch(reqs) == mbx.OK, be.last_error()
            bs = be.last_batch_stats.as_dict()
            assert bs["kernel_launches"] > 0 and bs["samples"] > 0
            for v, a, b in zip(vs, single, reqs):
                assert np.array_equal(a.escape_iteration, b.escape_iteration), (rep, v["label"])
                assert np.array_equal(a.iterations.view(np.uint32), b.iterations.view(np.uint32)), (rep, v["label"])
        print("\n[c3 subset] 8 views (%d supersampled), batch identical to single-view renders on two calls; shared passes %.2f ms"
              % (sum(v["sub"] > 1 for v in vs), bs["pass_gpu_ms"]))
    finally:
        be.close()
