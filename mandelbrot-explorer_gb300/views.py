"""Seeded synthetic views for the benchmark workloads and parity cases.

The reference publishes no dataset; its benchmarks are view coordinates. These
generators produce the view shapes the workloads are quoted on from recorded
seeds, as decimal strings consumable by the C ABI (and by the reference's own
tools): centre real/imaginary parts and the mpf ``scale`` (half-width 2/scale).
"""
from __future__ import annotations

import numpy as np

# Seahorse-valley centre of the plain FP64 workload (1280x720, half-width 1e-30).
C1_BASE_RE = "-0.743643887037151"
C1_BASE_IM = "0.131825904205330"


def extend_digits(base: str, total_significant: int, rng: np.random.RandomState) -> str:
    """Append seed-drawn decimal digits to ``base`` until it carries
    ``total_significant`` significant digits after the decimal point."""
    sign = "-" if base.startswith("-") else ""
    body = base.lstrip("-")
    intpart, frac = body.split(".")
    have = len(frac.lstrip("0")) if intpart == "0" else len(intpart) + len(frac)
    extra = max(0, total_significant - have)
    digits = "".join(str(d) for d in rng.randint(0, 10, size=extra))
    return sign + intpart + "." + frac + digits


def c1_view(seed: int = 1):
    """Plain FP64 workload: centre extended to 120 digits, half-width 1e-30
    (scale 2e30), maxiter 50000, bailout 2^8."""
    rng = np.random.RandomState(seed)
    cre = extend_digits(C1_BASE_RE, 120, rng)
    cim = extend_digits(C1_BASE_IM, 120, rng)
    return {"center_re": cre, "center_im": cim, "scale": "2" + "0" * 30, "max_iterations": 50000, "bailout": 256.0}
