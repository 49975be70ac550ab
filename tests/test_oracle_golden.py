"""The oracle against the reference engine's own output and its golden truth.

ref_*.f32 were rendered by the reference engine itself (compiled in place, see
tests/golden/make_golden.py); the oracle must reproduce them bit for bit on the
machine that produced them (x86-64 glibc). truth_*.f32 are the reference's own
arbitrary-precision golden files; the oracle must meet the tolerances the
reference's verify harness applies to its engine (src/tools/verify.cpp:11788-11890).
"""
import platform

import numpy as np
import pytest

import oracle
from conftest import load_cases, load_fixture

CASES = load_cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_build(name):
    c = CASES[name]
    it, nr, en, st = oracle.render(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"])
    ref_it, ref_nr = load_fixture(name, c)
    # Class is always exact; values are bit-exact on the fixture's own platform.
    assert np.array_equal(ref_it < -1.5, it < -1.5)
    assert np.array_equal(ref_it == -10.0, it == -10.0)
    if platform.machine() in ("x86_64", "AMD64"):
        assert np.array_equal(ref_it.view(np.uint32), it.view(np.uint32)), "oracle differs from the reference build"
        if ref_nr is not None:
            assert np.array_equal(ref_nr.view(np.uint32), nr.view(np.uint32))
    else:  # libm log may differ in the last ulp across architectures
        np.testing.assert_allclose(it, ref_it, rtol=1e-6, atol=0)
    # Escape iteration consistency with the smooth value (non-EDE frames).
    # (the stripe average and trap values are not escape counts)
    if not (c["coloring_method"] & (2 | 8 | 32)):
        ext = en > 0
        mu = it[ext].astype(np.float64)
        L = np.log2(np.log2(np.float64(np.float32(c["bailout"]))))
        gap = en[ext] - mu
        tol = 1e-3 + 2.0 * np.spacing(np.abs(it[ext])).astype(np.float64)  # float32 resolution of mu
        assert np.all(gap > L - tol) and np.all(gap < L + 1 + tol)


TRUTH_TOL = {  # verify.cpp:11837-11881, 307-388
    "point31": dict(maxdiff=12000.0, mean=200.0, p99=4000.0),
    "slowpoint": dict(maxdiff=90000.0, mean=300.0, p99=3000.0),
    "minibrot875": dict(maxdiff=1.0),
    "extref875": dict(maxdiff=1.0),
    "gui875": dict(maxdiff=1.0),
}


@pytest.mark.parametrize("name", sorted(TRUTH_TOL))
def test_oracle_meets_reference_truth(name):
    import os
    from conftest import GOLDEN

    c = CASES[name]
    it, _, _, _ = oracle.render(c["center_re"], c["center_im"], c["scale"], c["width"], c["height"], c["max_iterations"], sub=c["sub"], coloring_method=c["coloring_method"], bailout=c["bailout"])
    truth = np.fromfile(os.path.join(GOLDEN, "truth_%s.f32" % name), dtype="<f4")
    assert truth.size == it.size
    sampled = truth != -10.0 if name != "gui875" else it != -10.0
    if name == "gui875":
        W, H, S = c["width"], c["height"], c["sub"]
        base = np.zeros((H * S, W * S), bool)
        base[S // 2 :: S, S // 2 :: S] = True
        assert np.all(it.reshape(H * S, W * S)[base] != -10.0)
        assert np.sum(sampled & ~base.ravel()) > 0
    e_int, t_int = it < -1.5, truth < -1.5
    assert np.sum((e_int != t_int) & sampled) == 0, "class mismatch against the reference truth"
    both_ext = sampled & ~e_int & ~t_int
    d = np.abs(it[both_ext].astype(np.float64) - truth[both_ext])
    tol = TRUTH_TOL[name]
    assert d.max(initial=0.0) <= tol["maxdiff"]
    if "mean" in tol:
        assert d.mean() <= tol["mean"]
        assert np.sort(d)[int(np.ceil(0.99 * d.size)) - 1] <= tol["p99"]


JULIA = __import__("conftest").load_julia_cases()


@pytest.mark.parametrize("name", sorted(JULIA))
def test_oracle_julia_matches_reference_build(name):
    from conftest import load_julia_fixture

    c = JULIA[name]
    it, en = oracle.julia(c["center_re"], c["center_im"], c["scale"], c["fixed_c_re"], c["fixed_c_im"], c["width"], c["height"], c["max_iterations"], c["coloring_method"], c["bailout"], c.get("full_height", 0), c.get("row_base", 0))
    ref = load_julia_fixture(name)
    assert np.array_equal(ref < -1.5, it < -1.5)
    assert np.array_equal(en < 0, it < -1.5)
    if platform.machine() in ("x86_64", "AMD64"):
        assert np.array_equal(ref.view(np.uint32), it.view(np.uint32)), "oracle differs from the reference build"
    else:
        np.testing.assert_allclose(it, ref, rtol=1e-6, atol=0)


@pytest.mark.parametrize("label", ["1e-300", "1e-1000", "1e-1000-minibrot"])
def test_truth_subsets_reproduce(label):
    """The committed arbitrary-precision truth subsets of the 1080p deep frames
    (tests/golden/make_truth.py) are what the oracle's per-sample GMP iteration
    gives: a few of their samples recomputed, N exact, value within 1e-6."""
    import views
    from conftest import load_truth

    tr = load_truth(label)
    if tr is None:
        pytest.skip("truth subset not made")
    idx, tn, tv = tr
    assert idx.size == 4096 and np.all(np.diff(idx) > 0)
    # six samples spread over the subset, or for frames with long orbits the
    # six cheapest escaping ones (each GMP orbit at 3400 bits costs ~20 us per iteration)
    pick = np.arange(0, idx.size, idx.size // 6)[:6]
    if np.abs(tn[pick]).max() > 50000:
        pick = np.sort(np.argsort(np.where(tn > 0, tn, 1 << 30))[:6])
    v = views.frame(label)
    keys = np.stack([idx[pick] // 1920, idx[pick] % 1920, np.zeros(pick.size, int), np.zeros(pick.size, int)], axis=1)
    got_v, got_n = oracle.truth(v["center_re"], v["center_im"], v["scale"], 1920, 1080, v["max_iterations"], keys, bailout=v["bailout"])
    assert np.array_equal(got_n, tn[pick])
    np.testing.assert_allclose(got_v, tv[pick], rtol=1e-6, atol=0)
