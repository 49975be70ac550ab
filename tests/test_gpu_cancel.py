"""Cooperative cancellation (the reference's SetHalt / IComputeBackend::cancel,
mp.cpp:4342-4345, compute_backend.cpp:119-128), exercised from a second host
thread while the delta pass runs; the context must stay usable afterwards. No
GPU fault is involved: the kernels poll a host-mapped flag and return."""
import threading
import time

import numpy as np
import pytest

import mbx
from conftest import load_cases

pytestmark = pytest.mark.gpu


def test_cancel_from_other_thread_then_recover():
    be = mbx.create_compute_backend("cuda")
    try:
        c = load_cases()["deep51"]

        def req(w, h):
            return mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], w, h, c["max_iterations"], bailout=c["bailout"], reuse_reference=True)

        # A frame whose passes alone (reference resident) take long enough for
        # the cancel to land while a kernel runs: grow it until it does.
        full_s = 0.0
        for w, h in ((640, 480), (1280, 960), (2560, 1920)):
            assert be.compute_status(req(w, h)) == mbx.OK, be.last_error()  # builds the reference
            t0 = time.time()
            assert be.compute_status(req(w, h)) == mbx.OK, be.last_error()
            full_s = time.time() - t0
            if full_s >= 0.6:
                break
        assert full_s >= 0.6, "no frame long enough to cancel (%.3f s)" % full_s
        r = req(w, h)
        t = threading.Timer(full_s / 4, be.cancel)
        t0 = time.time()
        t.start()
        rc = be.compute_status(r)
        elapsed = time.time() - t0
        t.join()
        assert rc == mbx.E_CANCELLED
        # the kernels stop soon after the flag is set, well before the frame would end
        assert elapsed < full_s * 0.75, (elapsed, full_s)
        # cancelled until reset, like the reference's _cancelRequested
        small = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], 16, 12, 1000, bailout=c["bailout"])
        assert be.compute_status(small) == mbx.E_CANCELLED
        be.reset_cancellation()
        assert be.compute_status(small) == mbx.OK
        assert np.all(small.iterations != mbx.EMPTYPIXEL)
    finally:
        be.close()
