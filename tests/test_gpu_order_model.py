"""Learned ordering of the batched main pass (mbx_set_batch_scheduling).

* gradient check: the summed gradients of the tensor-core training kernels
  (tcgen05, minibatch rows spread over blocks) against the CPU reference
  (tests/order_ref.py) of the same BF16 MLP, over 256 and 384 rows;
* the learned-scheduling workload: 24 seed-drawn 256x256 tiles of the
  23040x12960 image (half-width 1e-500 at a minibrot's edge, maxiter 2e6) as
  one batch. The ordering changes no output (identical to the natural order in
  every mode), and the main FP32 pass that it orders is faster with the model
  than in the natural order (measured 81 -> 52.6 ms) and than with the
  untrained model, whose prediction is the tiles' mean probe cost (53.3 ms,
  min of two; three repeats of each differed by 0.1 ms): the trained model is
  the committed one (trained offline by order_train.py on the iteration maps
  of the 1e-30 view and the 1080p benchmark frames), trained further on this
  batch's own map.
"""
import numpy as np
import pytest

import mbx
import order_train
import views
from order_ref import SP, ref_gradient

pytestmark = pytest.mark.gpu


def test_gradient_matches_cpu_reference():
    be = mbx.create_compute_backend("cuda")
    rng = np.random.RandomState(7)
    for n in (256, 384):
        P = (rng.standard_normal(SP) * 0.2).astype(np.float32)
        X = rng.uniform(0.0, 1.0, (n, 24)).astype(np.float32)
        T = rng.uniform(0.0, 1.0, n).astype(np.float32)
        got = be.schedule_params(P)
        assert np.array_equal(got, P)
        g = be.schedule_gradient(X, T)
        r = ref_gradient(P, X, T, batch=n)
        for a, b in ((0, 1536), (1536, 1600), (1600, 5696), (5696, 5760), (5760, 5824), (5824, 5825)):
            scale = max(float(np.abs(r[a:b]).max()), 1e-6)
            assert float(np.abs(g[a:b] - r[a:b]).max()) <= 1e-4 * scale, (n, a, b)
        # no update happened
        assert np.array_equal(be.schedule_params(), P)
    be.close()


def _requests(tiles):
    return [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], v["width"], v["height"], v["max_iterations"], bailout=v["bailout"],
                               precision_bits=v["precision_bits"], precision_mode=mbx.PRECISION_MIXED, reference_re=v["reference_re"],
                               reference_im=v["reference_im"], reference_period=v["reference_period"]) for v in tiles]


def _run(be, tiles, k=2):
    """k renders of the batch: outputs of the last, min FP32-pass and graph ms."""
    f32, graph = [], []
    for _ in range(k):
        reqs = _requests(tiles)
        assert be.compute_batch(reqs) == mbx.OK, be.last_error()
        st = be.last_batch_stats.as_dict()
        f32.append(st["fp32_pass_gpu_ms"])
        graph.append(st["pass_gpu_ms"])
    return [(r.iterations.copy(), r.escape_iteration.copy()) for r in reqs], min(f32), min(graph)


def test_learned_order_on_c4_tiles():
    tiles = views.c4_tiles(n=24)
    init = order_train.initial_params(None)
    be = mbx.create_compute_backend("cuda")
    try:
        assert be.set_batch_scheduling(0) == mbx.OK
        _run(be, tiles, 1)  # the engines' orbits and tables
        base, nat_f32, nat_graph = _run(be, tiles)
        # untrained: the tiles in decreasing mean probe cost
        be.schedule_params(init)
        assert be.set_batch_scheduling(2) == mbx.OK, be.last_error()
        out, un_f32, un_graph = _run(be, tiles)
        for (it, en), (bit, ben) in zip(out, base):
            assert np.array_equal(en, ben) and np.array_equal(it, bit)
        # trained: the offline weights, trained further on this batch's map
        order_train.load_weights(be)
        assert be.set_batch_scheduling(1) == mbx.OK
        out, _, _ = _run(be, tiles, 1)
        for (it, en), (bit, ben) in zip(out, base):
            assert np.array_equal(en, ben) and np.array_equal(it, bit)
        assert be.set_batch_scheduling(2) == mbx.OK
        out, tr_f32, tr_graph = _run(be, tiles)
        for (it, en), (bit, ben) in zip(out, base):
            assert np.array_equal(en, ben) and np.array_equal(it, bit)
        print("\n[order 1e-500 tiles x24] FP32 pass: natural %.2f, untrained %.2f, trained %.2f ms; shared passes: %.1f, %.1f, %.1f ms"
              % (nat_f32, un_f32, tr_f32, nat_graph, un_graph, tr_graph))
        assert tr_f32 < 0.8 * nat_f32
        assert tr_f32 < un_f32
        assert tr_graph < nat_graph
    finally:
        be.close()
