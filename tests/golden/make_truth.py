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
       python tests/golden/make_truth.py --cases [case ...]  (full-frame truth of
       double-path parity cases, truthgen_<case>.npz; default: CASE_TRUTH)
       python tests/golden/make_truth.py --zoom  (zoom-sequence subsets, truth_zoom.npz)
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


# Double-path parity cases (tests/golden/cases.json, scale 1e6..1e280) that have
# no arbitrary-precision golden file from the reference: full-frame truth, so
# that forms which differ from the reference's double path on chaotic samples
# can be compared with it on the same footing (tests/test_gpu_mixed.py).
CASE_TRUTH = ("c1", "flake", "ticktock", "deep51")
# DE-coloured parity cases: truth of the distance (EDE and DE-overlay cases:
# oracle.truth with EDE, the reference's point routine) or of the normal-map
# angle arg z - arg dz/dc (the oracle's truth extension), for every sample in
# the reference's getIndex layout.
DE_CASE_TRUTH = ("c1_ede", "c1_normal", "c1_deovl_ss3", "minibrot875_ede", "minibrot875_normal", "exterior1000_deovl", "exterior1000_normal")


def case_path(name):
    return os.path.join(HERE, "truthgen_%s.npz" % name)


def make_case(name):
    import json

    c = json.load(open(os.path.join(HERE, "cases.json")))[name]
    W, H, sub = c["width"], c["height"], c["sub"]
    # every sample in getIndex order: sample row y = row sub + sub/2 + subrow
    ys, xs = np.meshgrid(np.arange(H * sub), np.arange(W * sub), indexing="ij")
    ys, xs = ys.ravel(), xs.ravel()
    keys = np.stack([ys // sub, xs // sub, ys % sub - sub // 2, xs % sub - sub // 2], axis=1)
    cm = c["coloring_method"] & (2 | 16 | 64)
    cm = 2 if cm & (2 | 64) else cm  # distance truth for EDE and the DE overlay
    t = time.time()
    tv, tn = oracle.truth(c["center_re"], c["center_im"], c["scale"], W, H, c["max_iterations"], keys, sub=sub, coloring_method=cm, bailout=c["bailout"], threads=os.cpu_count())
    np.savez_compressed(case_path(name), N=tn.astype(np.int32), value=tv.astype(np.float32))
    print("%s: %d samples in %.0f s, %d interior" % (name, keys.shape[0], time.time() - t, int(np.sum(tn < 0))))


# Zoom sequence (zoom.py): for the frames the GPU test renders (240x136), a
# seeded subset of 48 samples each with its exterior distance (EDE) and escape
# iteration (truth_zoom.npz: for each frame k, idx_k, N_k, value_k).
ZOOM_FRAMES = (8, 150, 300, 450, 599)
ZOOM_W, ZOOM_H = 240, 136


def make_zoom():
    import zoom

    out = {}
    t = time.time()
    for k in ZOOM_FRAMES:
        q = zoom.request(k, ZOOM_W, ZOOM_H)
        idx = np.sort(np.random.RandomState(700 + k).choice(ZOOM_W * ZOOM_H, size=48, replace=False))
        keys = np.stack([idx // ZOOM_W, idx % ZOOM_W, np.zeros_like(idx), np.zeros_like(idx)], axis=1)
        tv, tn = oracle.truth(q.center_re, q.center_im, q.scale, ZOOM_W, ZOOM_H, q.max_iterations, keys, coloring_method=q.coloring_method, bailout=q.bailout,
                              threads=os.cpu_count(), precision_bits=q.precision_bits)
        out["idx_%d" % k], out["N_%d" % k], out["value_%d" % k] = idx.astype(np.int32), tn.astype(np.int32), tv.astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "truth_zoom.npz"), **out)
    print("zoom: %d frames x 48 samples in %.0f s" % (len(ZOOM_FRAMES), time.time() - t))


if __name__ == "__main__":
    args = sys.argv[1:]
    if args and args[0] == "--zoom":
        make_zoom()
    elif args and args[0] == "--cases":
        for name in args[1:] or (CASE_TRUTH + DE_CASE_TRUTH):
            make_case(name)
    else:
        for label in args or views.TRUTH_FRAMES:
            make(label)
