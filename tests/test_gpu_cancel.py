"""Cooperative cancellation (the reference's SetHalt / IComputeBackend::cancel,
mp.cpp:4342-4345, compute_backend.cpp:119-128), exercised from a second host
thread; the context must stay usable afterwards. No GPU fault is involved: the
kernels poll a host-mapped flag and return."""
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
        req = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], 640, 480, c["max_iterations"], bailout=c["bailout"])
        t = threading.Timer(0.5, be.cancel)
        t.start()
        t0 = time.time()
        rc = be.compute_status(req)
        t.join()
        assert rc in (mbx.E_CANCELLED, mbx.OK)
        if rc == mbx.E_CANCELLED:
            assert time.time() - t0 < 30
        # cancelled until reset, like the reference's _cancelRequested
        small = mbx.ComputeRequest(c["center_re"], c["center_im"], c["scale"], 16, 12, 1000, bailout=c["bailout"])
        assert be.compute_status(small) == mbx.E_CANCELLED
        be.reset_cancellation()
        assert be.compute_status(small) == mbx.OK
        assert np.all(small.iterations != mbx.EMPTYPIXEL)
    finally:
        be.close()
