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


# ---------------------------------------------------------------------------
# Deep frames: 1920x1080, maxiter 1e6, centred a seed-drawn 10^-(k+5) vector
# away from the Newton-refined nucleus of a period-p component (p = 14164, in
# [2000, 20000]) at half-widths 10^-300 and 10^-1000. The nucleus is stored in
# views_data.json (regenerate with ``python views.py --regenerate``).
import json
import math
import os
from decimal import Decimal, getcontext

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(HERE, "views_data.json")


def nucleus():
    with open(DATA) as f:
        return json.load(f)


def deep_view(k: int, seed: int = 2, width: int = 1920, height: int = 1080, max_iterations: int = 1_000_000, bailout: float = 256.0):
    d = nucleus()
    rng = np.random.RandomState(seed * 1000 + k)
    ang = rng.uniform(0.0, 2.0 * math.pi)
    getcontext().prec = len(d["nucleus_re"]) + 20
    off = Decimal(10) ** (-(k + 5))
    cre = Decimal(d["nucleus_re"]) + off * Decimal(repr(math.cos(ang)))
    cim = Decimal(d["nucleus_im"]) + off * Decimal(repr(math.sin(ang)))
    return {
        "center_re": format(cre, "f"),
        "center_im": format(cim, "f"),
        "scale": "2" + "0" * k,
        "width": width,
        "height": height,
        "max_iterations": max_iterations,
        "bailout": bailout,
        "label": "1e-%d" % k,
        "period": d["period"],
    }


def c2_views(seed: int = 2, width: int = 1920, height: int = 1080, max_iterations: int = 1_000_000):
    """The two precision-workload frames (half-widths 1e-300 and 1e-1000)."""
    return [deep_view(k, seed, width, height, max_iterations) for k in (300, 1000)]


# A 1e-1000 frame that holds a whole minibrot and its surroundings: the
# period-1331 nucleus found next to the Misiurewicz point c = i (a disk of
# radius 5e-501 there holds a minibrot of about (5e-501)^2, size 3.6e-1001, 18 %
# of the frame width), the view centred a seed-drawn 1e-1003 vector from it.
# Escape iterations of its exterior run from ~14,500 to ~575,000; ~8 % of the
# samples are interior.
def minibrot_view(seed: int = 1000, width: int = 1920, height: int = 1080, max_iterations: int = 1_000_000, bailout: float = 256.0):
    d = nucleus()["minibrot1000"]
    rng = np.random.RandomState(seed)
    ang = rng.uniform(0.0, 2.0 * math.pi)
    getcontext().prec = len(d["nucleus_re"]) + 20
    off = Decimal(10) ** -1003
    cre = Decimal(d["nucleus_re"]) + off * Decimal(repr(math.cos(ang)))
    cim = Decimal(d["nucleus_im"]) + off * Decimal(repr(math.sin(ang)))
    return {
        "center_re": format(cre, "f"),
        "center_im": format(cim, "f"),
        "scale": "2" + "0" * 1000,
        "width": width,
        "height": height,
        "max_iterations": max_iterations,
        "bailout": bailout,
        "label": "1e-1000-minibrot",
        "period": d["period"],
    }


# The batching workload: 64 seed-drawn views of uneven shape — square sizes
# uniform over {256, 512, 1024, 2048, 4096}, log10 half-width uniform in
# [-600, -20], maxiter log-uniform in [1e4, 1e6], 3x3 adaptive supersampling
# (sub 3 with MBX_SUPER_SAMPLING) on a seed-drawn half of them — centred a
# seed-drawn vector of 0.3 half-widths from the zoom target nucleus (period
# 72852) so that every view holds structure. size_div divides the sizes (a
# stated sample of the workload).
def c3_views(seed: int = 3, n: int = 64, size_div: int = 1):
    d = nucleus()["zoom"]
    rng = np.random.RandomState(seed)
    ss = set(rng.permutation(n)[: n // 2].tolist())
    getcontext().prec = len(d["nucleus_re"]) + 20
    out = []
    for i in range(n):
        size = int(rng.choice([256, 512, 1024, 2048, 4096])) // size_div
        lhw = float(rng.uniform(20.0, 600.0))
        maxiter = int(round(10 ** rng.uniform(4.0, 6.0)))
        ang = rng.uniform(0.0, 2.0 * math.pi)
        hw = Decimal(10) ** Decimal(repr(-lhw))
        cre = Decimal(d["nucleus_re"]) + Decimal("0.3") * hw * Decimal(repr(math.cos(ang)))
        cim = Decimal(d["nucleus_im"]) + Decimal("0.3") * hw * Decimal(repr(math.sin(ang)))
        scale = Decimal(2) / hw
        out.append({
            "center_re": format(cre, "f"),
            "center_im": format(cim, "f"),
            "scale": format(scale.normalize(), "E").replace("E+", "e"),
            "width": size,
            "height": size,
            "sub": 3 if i in ss else 1,
            "coloring_method": 1 if i in ss else 0,
            "max_iterations": maxiter,
            "bailout": 256.0,
            "label": "c3-%02d" % i,
            "precision_bits": int(lhw * math.log2(10)) + 128,
        })
    return out


# Frames with committed arbitrary-precision truth subsets (tests/golden/make_truth.py).
TRUTH_FRAMES = ("1e-300", "1e-1000", "1e-1000-minibrot")


def frame(label: str, width: int = 1920, height: int = 1080):
    """A benchmark frame by label."""
    if label in ("1e-300", "1e-1000"):
        return deep_view(int(label[3:]), width=width, height=height)
    if label == "1e-1000-minibrot":
        return minibrot_view(width=width, height=height)
    raise KeyError(label)


if __name__ == "__main__":
    import sys

    if "--regenerate-zoom" in sys.argv:
        import mbx

        d = nucleus()
        getcontext().prec = len(d["nucleus_re"]) + 40
        rng = np.random.RandomState(5005)
        phi = rng.uniform(0, 2 * math.pi)
        r = Decimal(10) ** -850
        cre = Decimal(d["nucleus_re"]) + r * Decimal(repr(math.cos(phi)))
        cim = Decimal(d["nucleus_im"]) + r * Decimal(repr(math.sin(phi)))
        p, nre, nim, ls = mbx.find_nucleus(format(cre, "f"), format(cim, "f"), "3e-851", 200000, 3600)
        d["zoom"].update(nucleus_re=nre, nucleus_im=nim, period=p, size_log10=ls)
        json.dump(d, open(DATA, "w"), indent=1)
        print("period", p, "size 1e%.2f" % ls)
    if "--regenerate-minibrot" in sys.argv:
        import mbx

        rng = np.random.RandomState(21)
        phi = rng.uniform(0, 2 * math.pi)
        getcontext().prec = 1200
        dd = Decimal(10) ** -502
        p, nre, nim, ls = mbx.find_nucleus(format(dd * Decimal(repr(math.cos(phi))), "f"), format(1 + dd * Decimal(repr(math.sin(phi))), "f"), "5e-501", 400000, 3600)
        d = json.load(open(DATA))
        d["minibrot1000"].update(nucleus_re=nre, nucleus_im=nim, period=p, size_log10=ls)
        json.dump(d, open(DATA, "w"), indent=1)
        print("period", p, "size 1e%.2f" % ls)
    if "--regenerate" in sys.argv:
        import mbx

        cases = json.load(open(os.path.join(HERE, "..", "tests", "golden", "cases.json")))
        c = cases["minibrot875"]
        p, nre, nim, ls = mbx.find_nucleus(c["center_re"], c["center_im"], "1e-600", 100000, 3600)
        d = nucleus()
        d.update(nucleus_re=nre, nucleus_im=nim, period=p, size_log10=ls)
        json.dump(d, open(DATA, "w"), indent=1)
        print("period", p, "size 1e%.1f" % ls)
