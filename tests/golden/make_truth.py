"""Arbitrary-precision truth for seeded sample subsets of the 1080p deep frames.

For each named frame, a seeded subset of 4096 samples of the 1920x1080 grid is
iterated directly in arbitrary precision by the oracle (oracle.truth: the
reference's per-pixel GMP iteration accuratePointCompute, mp.cpp:719-894, at
the frame's precision). The escape iteration and smooth value of each sample
are written to truth_<frame>.npz (idx, N, value). The mixed-precision form is
held to these vectors by tests/test_gpu_truth.py and bench.py's accuracy
figures; recomputing them takes minutes of GMP work per frame, so they travel
with the repository.

Usage: python tests/golden/make_truth.py [frame ...]   (default: every frame)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "mandelbrot-explorer_gb300"), os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402
import views  # noqa: E402

W, H = 1920, 1080
SUBSET = 4096


def subset(label):
    """Sorted flat sample indices of a frame's seeded truth subset."""
    seed = {"1e-300": 4396, "1e-1000": 5096}.get(label, 6096)
    rng = np.random.RandomState(seed)
    return np.sort(rng.choice(W * H, size=SUBSET, replace=False))


def path(label):
    return os.path.join(HERE, "truth_c2_%s.npz" % label)


def load(label):
    """(idx, N, value) of a frame's committed truth subset, or None."""
    p = path(label)
    if not os.path.exists(p):
        return None
    z = np.load(p)
    return z["idx"], z["N"], z["value"]


def make(label):
    v = views.frame(label)
    idx = subset(label)
    keys = np.stack([idx // W, idx % W, np.zeros_like(idx), np.zeros_like(idx)], axis=1)
    t = time.time()
    tv, tn = oracle.truth(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], keys, bailout=v["bailout"], threads=os.cpu_count())
    np.savez_compressed(path(label), idx=idx.astype(np.int32), N=tn.astype(np.int32), value=tv.astype(np.float32))
    print("%s: %d samples in %.0f s, %d interior, N %d..%d" % (label, SUBSET, time.time() - t, int(np.sum(tn < 0)), int(tn[tn > 0].min(initial=0)), int(tn.max())))


if __name__ == "__main__":
    for label in sys.argv[1:] or views.TRUTH_FRAMES:
        make(label)
