"""Offline training of the batched passes' ordering model on the renderer's own
iteration maps, and loading of the trained weights.

The model (csrc/order_model.cu) predicts each 16x16 tile's mean FP32-lane cost
from the probe pass. Training renders a fixed set of frames through
mbx_compute_batch in scheduling mode 1: after each batch's passes the tensor-core
kernels train on the tiles' measured costs (32 Adam steps a batch). The frames:
the plain FP64 workload's view (1280x720, half-width 1e-30, maxiter 5e4) and the
precision workload's 1920x1080 frames at half-widths 1e-300 and 1e-1000 (plus the
1e-1000 frame holding a minibrot), all in the mixed form.

    python order_train.py [--batches N] [--out order_model_params.npz]

The committed weights (order_model_params.npz) were made by this script; the
scheduling tests and the benchmark load them with load_weights().
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

import mbx
import views

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "order_model_params.npz")


def training_requests():
    """The training frames as mixed-form requests."""
    c1 = views.c1_view()
    out = [mbx.ComputeRequest(c1["center_re"], c1["center_im"], c1["scale"], 1280, 720, c1["max_iterations"], bailout=c1["bailout"],
                              precision_mode=mbx.PRECISION_MIXED)]
    for label in ("1e-300", "1e-1000", "1e-1000-minibrot"):
        v = views.frame(label)
        out.append(mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], v["width"], v["height"], v["max_iterations"],
                                      bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED))
    return out


def train(be: mbx.CudaComputeBackend, batches: int = 8, log=print):
    """Train from the initial weights over `batches` renders of the training
    frames; returns the parameters."""
    be.schedule_params(initial_params(be))
    if be.set_batch_scheduling(1) != mbx.OK:
        raise RuntimeError(be.last_error())
    for b in range(batches):
        t = time.time()
        if be.compute_batch(training_requests()) != mbx.OK:
            raise RuntimeError(be.last_error())
        log("batch %d: %.2f s" % (b, time.time() - t))
    be.set_batch_scheduling(0)
    return be.schedule_params()


_INITIAL = None


def initial_params(be=None):
    """The untrained model's parameters: a fresh context's initial ones (read
    once per process)."""
    global _INITIAL
    if _INITIAL is None:
        fresh = mbx.create_compute_backend("cuda")
        try:
            _INITIAL = fresh.schedule_params().copy()
        finally:
            fresh.close()
    return _INITIAL


def load_weights(be: mbx.CudaComputeBackend, path: str = WEIGHTS) -> np.ndarray:
    """Set the committed trained weights on a context."""
    p = np.load(path)["params"].astype(np.float32)
    be.schedule_params(p)
    return p


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--batches", type=int, default=8)
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args()
    be = mbx.create_compute_backend("cuda")
    p = train(be, a.batches)
    be.close()
    np.savez(a.out, params=p, batches=a.batches, steps_per_batch=32,
             frames="c1 1280x720; 1e-300, 1e-1000, 1e-1000-minibrot 1920x1080 (mixed form)")
    print("wrote", a.out)
