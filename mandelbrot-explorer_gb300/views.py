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
from decimal import Context, Decimal, getcontext

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


# The learned-scheduling workload: a 7680x4320 image with uniform 3x3
# supersampling, rendered as 23040x12960 samples with sub 1; half-width 1e-500,
# maxiter 2e6. Its minibrot is the period-38045 nucleus stored in
# views_data.json ("c4", size 3.2e-501: the minibrot spans about a third of
# the view's width; it is the copy of the standard set's period-5 real-axis
# minibrot inside a period-7609
# minibrot found by a seeded search next to the period-14164 nucleus of the
# deep frames). The view is
# centred 1e-3 of the view width outward from a point of that minibrot's edge:
# the boundary pixel nearest a seed-drawn point of the estimated main cardioid
# (nucleus + size (e/2 - e^2/4)), refined by renders at shrinking half-widths
# (c4_edge_search, which needs a GPU), so the edge crosses the image near its
# centre.
C4_W, C4_H, C4_HW_LOG10, C4_MXIT = 23040, 12960, -500, 2_000_000


def c4_cardioid_point(seed: int = 4):
    """Estimated edge point: nucleus + size (e/2 - e^2/4), e = exp(i th) with
    th seed-drawn away from the cusp."""
    d = nucleus()["c4"]
    rng = np.random.RandomState(seed)
    th = rng.uniform(0.25 * math.pi, 1.75 * math.pi)
    getcontext().prec = len(d["nucleus_re"]) + 20
    sre, sim = Decimal(d["size_re"]), Decimal(d["size_im"])
    e = complex(math.cos(th), math.sin(th))
    card = e / 2 - e * e / 4
    ere = Decimal(d["nucleus_re"]) + sre * Decimal(repr(card.real)) - sim * Decimal(repr(card.imag))
    eim = Decimal(d["nucleus_im"]) + sre * Decimal(repr(card.imag)) + sim * Decimal(repr(card.real))
    return ere, eim


def c4_view():
    """Centre, half-width and pitch of the whole learned-scheduling image (decimals)."""
    d = nucleus()["c4"]
    getcontext().prec = len(d["nucleus_re"]) + 20
    hw = Decimal(10) ** C4_HW_LOG10
    nx, ny = d["edge_normal"]
    cre = Decimal(d["edge_re"]) + Decimal("1e-3") * 2 * hw * Decimal(repr(nx))
    cim = Decimal(d["edge_im"]) + Decimal("1e-3") * 2 * hw * Decimal(repr(ny))
    return {"center_re": cre, "center_im": cim, "hw": hw, "pitch": 2 * hw / (C4_W - 1), "width": C4_W, "height": C4_H,
            "max_iterations": C4_MXIT, "bailout": 256.0, "period": d["period"]}


def c4_edge_search(be, seed: int = 4, n: int = 512, levels: int = 8):
    """The boundary of the learned-scheduling image's minibrot near its seed-drawn cardioid point:
    render n x n at maxiter 2e6 around the current point, take the boundary
    pixel (non-escaping, with an escaping 4-neighbour) nearest it, divide the
    half-width by 32, repeat down to a half-width below 1e-502. Returns the
    edge point and its outward normal (exterior minus interior pixel means in
    a 9x9 window)."""
    import mbx

    d = nucleus()["c4"]
    getcontext().prec = len(d["nucleus_re"]) + 20
    sre, sim = Decimal(d["size_re"]), Decimal(d["size_im"])
    tre, tim = c4_cardioid_point(seed)
    cre, cim = Decimal(d["nucleus_re"]), Decimal(d["nucleus_im"])
    hw = 2 * (sre * sre + sim * sim).sqrt()
    res = None
    for _ in range(levels):
        scale = format(Context(prec=30).divide(Decimal(2), hw), "E").replace("E+", "e")
        r = mbx.ComputeRequest(format(cre, "f"), format(cim, "f"), scale, n, n, C4_MXIT, bailout=256.0, precision_bits=2000,
                               precision_mode=mbx.PRECISION_MIXED, reference_re=d["nucleus_re"], reference_im=d["nucleus_im"],
                               reference_period=d["period"])
        if be.compute_status(r) != mbx.OK:
            raise RuntimeError(be.last_error())
        it = r.iterations.reshape(n, n)
        inside = (it < 0) | (it >= C4_MXIT - 1)
        pitch = 2 * hw / (n - 1)
        c0re, c0im = cre - hw, cim - hw
        out = np.zeros_like(inside)
        out[1:, :] |= ~inside[:-1, :]
        out[:-1, :] |= ~inside[1:, :]
        out[:, 1:] |= ~inside[:, :-1]
        out[:, :-1] |= ~inside[:, 1:]
        bd = np.argwhere(inside & out)
        if len(bd) == 0:
            break
        tx, ty = float((tre - c0re) / pitch), float((tim - c0im) / pitch)
        py, px = bd[np.argmin((bd[:, 1] - tx) ** 2 + (bd[:, 0] - ty) ** 2)]
        cre, cim = c0re + pitch * Decimal(int(px)), c0im + pitch * Decimal(int(py))
        tre, tim = cre, cim
        y0, y1, x0, x1 = max(0, py - 4), min(n, py + 5), max(0, px - 4), min(n, px + 5)
        yy, xx = np.mgrid[y0:y1, x0:x1]
        w = inside[y0:y1, x0:x1]
        v = np.array([xx[~w].mean() - xx[w].mean(), yy[~w].mean() - yy[w].mean()])
        v = v / np.linalg.norm(v)
        res = dict(edge_re=format(cre, "f"), edge_im=format(cim, "f"), edge_normal=[float(v[0]), float(v[1])],
                   edge_pitch_log10=float(pitch.log10()))
        if float(hw.log10()) < C4_HW_LOG10 - 2:
            break
        hw = hw / 32
    return res


def c4_tiles(seed: int = 4, n: int = 32, tile: int = 256):
    """n seed-drawn tile x tile tiles of the learned-scheduling image (without repeats), each a
    view with the image's pixel pitch, its centre at the tile's centre. Every
    tile names the image's minibrot nucleus as its periodic reference (one orbit for all)."""
    v = c4_view()
    d = nucleus()["c4"]
    getcontext().prec = len(d["nucleus_re"]) + 20
    nx, ny = C4_W // tile, C4_H // tile
    rng = np.random.RandomState(seed)
    picks = rng.permutation(nx * ny)[:n]
    p = v["pitch"]
    # pixel (x, y) of the image sits at c0 + x pitch + i y pitch
    c0re = v["center_re"] - p * Decimal(C4_W - 1) / 2
    c0im = v["center_im"] - p * Decimal(C4_H - 1) / 2
    hw_t = p * Decimal(tile - 1) / 2
    scale = format(Context(prec=30).divide(Decimal(2), hw_t), "E").replace("E+", "e")
    out = []
    for k in picks.tolist():
        ty, tx = divmod(int(k), nx)
        cre = c0re + p * (Decimal(tx * tile) + Decimal(tile - 1) / 2)
        cim = c0im + p * (Decimal(ty * tile) + Decimal(tile - 1) / 2)
        out.append({
            "center_re": format(cre, "f"),
            "center_im": format(cim, "f"),
            "scale": scale,
            "width": tile,
            "height": tile,
            "max_iterations": C4_MXIT,
            "bailout": 256.0,
            "precision_bits": int(-C4_HW_LOG10 * math.log2(10)) + 128,
            "reference_re": d["nucleus_re"],
            "reference_im": d["nucleus_im"],
            "reference_period": d["period"],
            "label": "c4-%d-%d" % (tx, ty),
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
    if "--regenerate-c4" in sys.argv:
        import mbx
        import mpmath

        def complex_size(nre, nim, p):
            """1 / (beta lambda^2) over one period."""
            mpmath.mp.prec = 2400
            c = mpmath.mpc(mpmath.mpf(nre), mpmath.mpf(nim))
            z, lam, beta = mpmath.mpc(0), mpmath.mpc(1), mpmath.mpc(1)
            for _ in range(1, p):
                z = z * z + c
                lam = 2 * z * lam
                beta = beta + 1 / lam
            s = 1 / (beta * lam * lam)
            return mpmath.nstr(s.real, 20), mpmath.nstr(s.imag, 20)

        d = nucleus()
        getcontext().prec = len(d["nucleus_re"]) + 40
        rng = np.random.RandomState(4004)
        phi = rng.uniform(0, 2 * math.pi)
        r = Decimal(10) ** -250
        cre = Decimal(d["nucleus_re"]) + r * Decimal(repr(math.cos(phi)))
        cim = Decimal(d["nucleus_im"]) + r * Decimal(repr(math.sin(phi)))
        p, nre, nim, ls = mbx.find_nucleus(format(cre, "f"), format(cim, "f"), "3e-251", 200000, 2400)
        sre, sim = complex_size(nre, nim, p)
        parent = dict(nucleus_re=nre, nucleus_im=nim, period=p, size_log10=ls, size_re=sre, size_im=sim)
        # the parent's copy of the period-5 minibrot on the real axis of the standard set
        x = Decimal("-1.985424253054205")
        cre = Decimal(nre) + Decimal(sre) * x
        cim = Decimal(nim) + Decimal(sim) * x
        mag = (Decimal(sre) ** 2 + Decimal(sim) ** 2).sqrt()
        p, nre, nim, ls = mbx.find_nucleus(format(cre, "f"), format(cim, "f"), format(mag * Decimal("1e-4"), "E"), 400000, 2400)
        sre, sim = complex_size(nre, nim, p)
        d["c4"] = dict(nucleus_re=nre, nucleus_im=nim, period=p, size_log10=ls, size_re=sre, size_im=sim, parent=parent)
        json.dump(d, open(DATA, "w"), indent=1)
        print("period", p, "size 1e%.2f" % ls)
    if "--regenerate-c4-edge" in sys.argv:
        import mbx

        be = mbx.create_compute_backend("cuda")
        d = nucleus()
        d["c4"].update(c4_edge_search(be))
        be.close()
        json.dump(d, open(DATA, "w"), indent=1)
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
