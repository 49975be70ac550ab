"""The zoom sequence's frame parameters (no GPU): geometric half-widths from 1
to 1e-1000 and maxiter from 1e3 to 5e6 over 600 frames, every frame centred on
the stored period-72852 target nucleus."""
from decimal import Decimal

import zoom


def test_frame_parameters():
    s0, m0 = zoom.frame_params(0)
    s1, m1 = zoom.frame_params(599)
    assert Decimal(s0) == 2 and m0 == 1000
    assert Decimal(s1) == Decimal("2e1000") and m1 == 5_000_000
    prev = Decimal(0)
    for k in range(0, 600, 37):
        s, m = zoom.frame_params(k)
        assert Decimal(s) > prev
        prev = Decimal(s)
    re, im, p = zoom.target()
    assert 10000 <= p <= 100000
    q = zoom.request(300, 64, 36)
    assert q.reference_period == p and q.center_re == re and q.precision_bits >= 3400
