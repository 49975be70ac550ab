"""Benchmark: 1080p deep-zoom frames, tuned (mixed-precision) form vs the plain
FP64 GPU form, at accuracy, with the reference path's CPU restatement timed on
the host cores beside them.

Workload (one step): three 1920x1080 frames at maxiter 1e6, bailout 2^8 — the
two precision frames, half-widths 1e-300 and 1e-1000 centred a seed-drawn
1e-(k+5) vector from the Newton-refined period-14164 nucleus (views.c2_views;
read literally, the first is all exterior and the second all interior), and a
1e-1000 frame holding a whole period-1331 minibrot with its surroundings
(views.minibrot_view: exterior escape iterations ~14,500 to ~575,000, 8 %
interior). Inputs are synthetic seeded views; the reference publishes no
dataset.

  value  : effective pixel-iterations (sum of N, maxiter for interior) per second
           of the tuned form through the C ABI with device-resident outputs and
           the per-frame reference orbit/BLA resident (reuse_reference).
  e2e    : the same metric through the C ABI with host buffers and a fresh
           reference build (GMP orbit, nucleus search, uploads, D2H) per frame.
  plain  : the exact FP64 GPU form (reference operation order) on the same frames.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank renders its own replica of the workload (the frames
are independent; no collective is needed) and rank 0 reports.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "mandelbrot-explorer_gb300"))

import numpy as np  # noqa: E402

METRIC = "1080p deep-zoom frame ms & Gpixel-iter/s: tuned form vs plain FP64 GPU, at accuracy"
UNIT = "Gpixel-iter/s"
FLOPS_PER_STEP = 25  # mp.cpp:2457-2469 + rebase test :2558 (an FMA counts 2)
FLOPS_PER_BLA = 19   # mp.cpp:2732-2740


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons), "samples": len(sm)}


def render(be, mbx, v, mode, device_out=None, reuse=False, width=None, height=None):
    W = width or v["width"]
    H = height or v["height"]
    kw = {}
    if device_out is not None:
        kw = dict(iterations=device_out[0], escape_iteration=device_out[1])
    req = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], bailout=v["bailout"], precision_mode=mode, reuse_reference=reuse, **kw)
    rc = be.compute_status(req)
    if rc != mbx.OK:
        raise RuntimeError("render failed (%d): %s" % (rc, be.last_error()))
    return req, be.last_stats.as_dict()


def cpu_reference(views_list, sample_w, sample_h, threads):
    """The reference path's CPU restatement (oracle port) on a bounded sample:
    the same views rendered at sample_w x sample_h (same view region, fewer
    pixels); returns (Gpixel-iter/s, seconds, effective iterations)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    eff = 0
    t0 = time.perf_counter()
    for v in views_list:
        it, _, en, _ = oracle.render(v["center_re"], v["center_im"], v["scale"], sample_w, sample_h, v["max_iterations"], bailout=v["bailout"], threads=threads)
        eff += int(np.where(en > 0, en, v["max_iterations"]).astype(np.int64).sum())
    dt = time.perf_counter() - t0
    return eff / dt / 1e9, dt, eff


def profile_c4(args):
    """args.profile_c4 tiles of the learned-scheduling image (256x256 each) as
    one batch, warmup + steps times, the model ordering and training (probe
    cells, prediction, ordering, shared passes, tcgen05 training)."""
    import mbx
    import order_train
    import views

    tiles = views.c4_tiles(n=args.profile_c4)
    be = mbx.create_compute_backend("cuda")
    order_train.load_weights(be)
    assert be.set_batch_scheduling(1) == mbx.OK, be.last_error()
    times = []
    for k in range(args.warmup + args.steps):
        reqs = [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], v["width"], v["height"], v["max_iterations"], bailout=v["bailout"],
                                   precision_bits=v["precision_bits"], precision_mode=mbx.PRECISION_MIXED, reference_re=v["reference_re"],
                                   reference_im=v["reference_im"], reference_period=v["reference_period"]) for v in tiles]
        t = time.perf_counter()
        assert be.compute_batch(reqs) == mbx.OK, be.last_error()
        if k >= args.warmup:
            times.append((time.perf_counter() - t) * 1e3)
    st = be.last_batch_stats.as_dict()
    be.close()
    print(json.dumps({"profile_c4": {"tiles": len(tiles), "ms": float(np.mean(times)), "shared_passes_gpu_ms": st["pass_gpu_ms"],
                                     "fp32_pass_gpu_ms": st["fp32_pass_gpu_ms"], "kernel_launches": st["kernel_launches"]}}))


def profile_run(args, vlist):
    """A small, fixed launch sequence for profilers: each listed view rendered
    warmup + steps times in the mixed form with the default launch shape and a
    resident reference; prints one JSON line of per-view frame times."""
    import mbx

    out = {}
    if args.profile_batch:
        # the views as one batch with the learned ordering training on each
        # batch (probe grid, prediction, bucket sort, shared passes, training)
        be = mbx.create_compute_backend("cuda")
        assert be.set_batch_scheduling(1) == mbx.OK, be.last_error()
        reqs = [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], args.width, args.height, v["max_iterations"], bailout=v["bailout"],
                                   precision_mode=mbx.PRECISION_MIXED, reuse_reference=True) for v in vlist]
        times = []
        for k in range(args.warmup + args.steps):
            t = time.perf_counter()
            assert be.compute_batch(reqs) == mbx.OK, be.last_error()
            if k >= args.warmup:
                times.append((time.perf_counter() - t) * 1e3)
        out["batch"] = {"ms": float(np.mean(times)), "shared_passes_gpu_ms": be.last_batch_stats.pass_gpu_ms}
        be.close()
        print(json.dumps({"profile": out, "resolution": "%dx%d" % (args.width, args.height)}))
        return
    for v in vlist:
        be = mbx.create_compute_backend("cuda")
        times = []
        for k in range(args.warmup + args.steps):
            t = time.perf_counter()
            req, st = render(be, mbx, v, mbx.PRECISION_EXACT if args.profile_exact else mbx.PRECISION_MIXED, reuse=True, width=args.width, height=args.height)
            # the render tool's image epilogue on the frame (host values, RGB back)
            be.colorize(req.iterations, args.width, args.height, mbx.ColorParams())
            if k >= args.warmup:
                times.append((time.perf_counter() - t) * 1e3)
        out[v["label"]] = {"frame_ms": float(np.mean(times)), "pass_gpu_ms": st["pass_gpu_ms"], "fp32_pass_gpu_ms": st["fp32_pass_gpu_ms"], "rerun_gpu_ms": st["rerun_gpu_ms"],
                           "exact_form_gpu_ms": st["rerun_fp64_gpu_ms"], "fp64_reruns": st["fp64_reruns"], "exact_reruns": st["exact_reruns"], "steps": st["steps"],
                           "bla_applies": st["bla_applies"], "fp32_pass_steps": st["fp32_pass_steps"], "fp32_pass_bla_applies": st["fp32_pass_bla_applies"],
                           "interior": st["interior"], "fp32_unvouched_interior": st["fp32_unvouched_interior"], "fp32_unvouched_escape": st["fp32_unvouched_escape"],
                           "rebases": st["rebases"], "exact_steps": st["exact_steps"], "fe_rebases": st["fe_rebases"],
                           "color_gpu_ms": be.last_color_stats()[0]}
        be.close()
    print(json.dumps({"profile": out, "resolution": "%dx%d" % (args.width, args.height)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--cpu-sample", default="960x540", help="cpu_baseline sample size (same views); one render of each")
    ap.add_argument("--ref-sample", default="960x540", help="--impl reference per-step sample size (same views)")
    ap.add_argument("--plain-sample", default="full", help="plain FP64 GPU sample size (same views), WxH or 'full' (the frames' own size)")
    ap.add_argument("--profile", default=None, help="comma-separated view labels (e.g. 1e-300): render (and colour) only those, default launch shape, no baselines (for ncu captures)")
    ap.add_argument("--profile-batch", action="store_true", help="with --profile: render the views as one batch with the learned ordering training")
    ap.add_argument("--profile-exact", action="store_true", help="with --profile: render the views in the exact form (MBX_PRECISION_EXACT)")
    ap.add_argument("--profile-c4", type=int, default=0, help="render N tiles of the learned-scheduling image as one batch with the model training on it (for ncu captures)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    import order_train
    import views

    if args.profile_c4:
        profile_c4(args)
        return

    vlist = views.c2_views(width=args.width, height=args.height) + [views.minibrot_view(width=args.width, height=args.height)]
    sw, sh = (int(x) for x in args.cpu_sample.split("x"))
    threads = os.cpu_count() or 1

    if args.profile:
        profile_run(args, [v for v in vlist if v["label"] in args.profile.split(",")])
        return

    if args.impl == "reference":
        if rank != 0:
            return
        sw, sh = (int(x) for x in args.ref_sample.split("x"))
        vals = []
        for _ in range(max(1, args.warmup // 3)):
            cpu_reference(vlist, sw // 2, sh // 2, threads)
        tot_t, tot_e = 0.0, 0
        for _ in range(args.steps):
            v, dt, eff = cpu_reference(vlist, sw, sh, threads)
            vals.append(v)
            tot_t += dt
            tot_e += eff
        value = tot_e / tot_t / 1e9
        line = {
            "impl": "reference",
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": args.gpus,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": tot_t / args.steps * 1e3,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "1080p deep frames 1e-300, 1e-1000 and 1e-1000 with a minibrot, sampled at %dx%d of the 1920x1080 views" % (sw, sh), "maxiter": 1000000, "bailout": 256},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": "the three views rendered at %dx%d (same view regions) per step by the oracle (CPU restatement of the reference path; the reference's AVX2 sources do not build on this Arm host)" % (sw, sh)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return

    import torch

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import mbx

    be = mbx.create_compute_backend("cuda", local)
    fp32_peak = be.measure_fma_peak(False)
    fp64_peak = be.measure_fma_peak(True)
    # one context per frame: each keeps its own resident reference orbit / BLA table,
    # and its launch shape picked by the autotuner on the frame itself (outside
    # the timed region)
    W, H = args.width, args.height
    ctxs = [mbx.create_compute_backend("cuda", local) for _ in vlist]
    tuning = {}
    for v, cx in zip(vlist, ctxs):
        calib = mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED)
        tuning[v["label"]] = cx.autotune(calib)
    n = W * H
    outs = [(torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.int32, device="cuda")) for _ in vlist]
    reruns = {}

    per_frame = {v["label"]: dict(eff=0, steps=0, bla=0, gpu_ms=0.0, fp32_ms=0.0, fp32_steps=0, fp32_bla=0, rerun_ms=0.0, exact_ms=0.0) for v in vlist}

    def step(reuse=True, record=False):
        eff = steps = bla = launches = 0
        gpu_ms = 0.0
        per_view = []
        for v, o, cx in zip(vlist, outs, ctxs):
            t = time.perf_counter()
            _, st = render(cx, mbx, v, mbx.PRECISION_MIXED, device_out=o, reuse=reuse)
            per_view.append((time.perf_counter() - t) * 1e3)
            eff += st["effective_iterations"]
            steps += st["steps"]
            bla += st["bla_applies"]
            launches += st["kernel_launches"]
            gpu_ms += st["pass_gpu_ms"]
            reruns[v["label"]] = {"double_float": st["fp64_reruns"], "exact_form": st["exact_reruns"]}
            if record:
                pf = per_frame[v["label"]]
                pf["eff"] += st["effective_iterations"]
                pf["steps"] += st["steps"]
                pf["bla"] += st["bla_applies"]
                pf["gpu_ms"] += st["pass_gpu_ms"]
                pf["fp32_ms"] += st["fp32_pass_gpu_ms"]
                pf["fp32_steps"] += st["fp32_pass_steps"]
                pf["fp32_bla"] += st["fp32_pass_bla_applies"]
                pf["rerun_ms"] += st["rerun_gpu_ms"]
                pf["exact_ms"] += st["rerun_fp64_gpu_ms"]
        return eff, steps, bla, launches, gpu_ms, per_view

    # warm-up (the first step builds each frame's reference)
    for _ in range(args.warmup):
        step(reuse=True)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tot = [0, 0, 0, 0, 0.0]
    frame_ms = np.zeros(len(vlist))
    for _ in range(args.steps):
        eff, steps, bla, launches, gpu_ms, per_view = step(reuse=True, record=True)
        tot[0] += eff
        tot[1] += steps
        tot[2] += bla
        tot[3] += launches
        tot[4] += gpu_ms
        frame_ms += np.array(per_view)
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    ms_per_step = elapsed / args.steps * 1e3
    value = tot[0] * world / elapsed / 1e9

    # the same frames through the batched API: the frames' passes in shared
    # launches (one CUDA graph), references resident
    bat = mbx.create_compute_backend("cuda", local)
    breqs = [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED,
                                reuse_reference=True, iterations=o[0], escape_iteration=o[1]) for v, o in zip(vlist, outs)]
    for _ in range(args.warmup):
        assert bat.compute_batch(breqs) == mbx.OK, bat.last_error()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b_eff, b_gpu = 0, 0.0
    for _ in range(args.steps):
        assert bat.compute_batch(breqs) == mbx.OK, bat.last_error()
        b_eff += bat.last_batch_stats.effective_iterations + sum(s.effective_iterations for s in bat.last_view_stats)
        b_gpu += bat.last_batch_stats.pass_gpu_ms
    torch.cuda.synchronize()
    b_elapsed = time.perf_counter() - t0
    batched = {"ms_per_step": b_elapsed / args.steps * 1e3, "value": b_eff / b_elapsed / 1e9, "unit": UNIT, "shared_passes_gpu_ms": b_gpu / args.steps,
               "note": "mbx_compute_batch: frames of 2^20 pixels or more (these three) render on their own streams as soon as their host work is done; smaller frames share one CUDA graph of probe, main and rerun passes; default launch shape"}
    # the learned-scheduled form: the cost model trains on the warm-up batches
    # (mode 1), then orders the timed ones (mode 2); outputs are identical
    ref_out = [o[1].clone() for o in outs]
    assert bat.set_batch_scheduling(1) == mbx.OK, bat.last_error()
    for _ in range(max(args.warmup, 3)):
        assert bat.compute_batch(breqs) == mbx.OK, bat.last_error()
    assert bat.set_batch_scheduling(2) == mbx.OK, bat.last_error()
    l_gpu = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert bat.compute_batch(breqs) == mbx.OK, bat.last_error()
        l_gpu += bat.last_batch_stats.pass_gpu_ms
    torch.cuda.synchronize()
    l_elapsed = time.perf_counter() - t0
    identical = all(bool(torch.equal(a, o[1])) for a, o in zip(ref_out, outs))
    batched["learned_order"] = {"ms_per_step": l_elapsed / args.steps * 1e3, "shared_passes_gpu_ms": l_gpu / args.steps, "identical_to_natural_order": identical}
    # each 1e-1000 frame alone in the learned-scheduled form (the stated target
    # compares a 1080p 1e-1000 frame in that form with the plain FP64 form)
    batched["learned_order"]["frame_ms"] = {}
    for q, v in zip(breqs, vlist):
        if not v["label"].startswith("1e-1000"):
            continue
        for _ in range(3):
            assert bat.compute_batch([q]) == mbx.OK, bat.last_error()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            assert bat.compute_batch([q]) == mbx.OK, bat.last_error()
        torch.cuda.synchronize()
        batched["learned_order"]["frame_ms"][v["label"]] = (time.perf_counter() - t0) / args.steps * 1e3
    bat.close()

    # image epilogue: the render tool's colouring (palette, gamma; ss 1) of each
    # resident 1080p frame on the device, values -> RGB8, timed by the
    # library's CUDA events around the kernel
    peaks_path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    hbm_peak = json.load(open(peaks_path)).get("hbm_gbs") if os.path.exists(peaks_path) else None
    hbm_src = "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_peak else "fallback 6800 GB/s"
    hbm_peak = hbm_peak or 6800.0
    col = ctxs[0]
    cparams = mbx.ColorParams()
    rgbs = [torch.empty((H, W, 3), dtype=torch.uint8, device="cuda") for _ in vlist]
    for _ in range(args.warmup):
        for o, r in zip(outs, rgbs):
            col.colorize(o[0], W, H, cparams, rgb=r)
    c_ms, c_fb, c_n = 0.0, 0, 0
    for _ in range(args.steps):
        for o, r in zip(outs, rgbs):
            col.colorize(o[0], W, H, cparams, rgb=r)
            ms_, fb_ = col.last_color_stats()
            c_ms, c_fb, c_n = c_ms + ms_, c_fb + fb_, c_n + 1
    c_per = c_ms / c_n
    c_bytes = W * H * (4 + 3)
    epilogue = {"kernel": "k_colorize", "ms_per_frame": c_per, "bytes_per_frame": c_bytes, "achieved_gbs": c_bytes / (c_per / 1e3) / 1e9,
                "hbm_peak_gbs": hbm_peak, "frac_hbm": c_bytes / (c_per / 1e3) / 1e9 / hbm_peak, "peak_source": hbm_src,
                "fp64_fallbacks_per_frame": c_fb / c_n,
                "note": "mbx_colorize on device values (log-power palette, ss 1): 4 B read + 3 B written per pixel; compute-bound on the pair-of-floats log/pow"}

    # end to end: host buffers, fresh reference per frame, D2H inside
    e2e_eff, e2e_t = 0, 0.0
    host_frames = []
    for v in vlist:
        t = time.perf_counter()
        req, st = render(be, mbx, v, mbx.PRECISION_MIXED, reuse=False)
        e2e_t += time.perf_counter() - t
        e2e_eff += st["effective_iterations"]
        host_frames.append(req.escape_iteration.copy())
    e2e_value = e2e_eff / e2e_t / 1e9
    # the same step (all frames) as one mbx_compute_batch call with host
    # buffers and fresh references: the frames' GMP work runs concurrently on
    # the host, their passes share one graph; D2H of every frame inside
    bat2 = mbx.create_compute_backend("cuda", local)
    b_reqs = [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED) for v in vlist]
    assert bat2.compute_batch(b_reqs) == mbx.OK, bat2.last_error()  # allocations
    eb_eff, eb_t, h2d, d2h = 0, 0.0, 0, 0
    for _ in range(2):
        b_reqs = [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], W, H, v["max_iterations"], bailout=v["bailout"], precision_mode=mbx.PRECISION_MIXED) for v in vlist]
        t = time.perf_counter()
        assert bat2.compute_batch(b_reqs) == mbx.OK, bat2.last_error()
        eb_t += time.perf_counter() - t
        eb_eff += bat2.last_batch_stats.effective_iterations + sum(s_.effective_iterations for s_ in bat2.last_view_stats)
        # bytes the library copied in this step, counted at each copy
        h2d += bat2.last_batch_stats.h2d_bytes + sum(s_.h2d_bytes for s_ in bat2.last_view_stats)
        d2h += bat2.last_batch_stats.d2h_bytes + sum(s_.d2h_bytes for s_ in bat2.last_view_stats)
    h2d //= 2
    d2h //= 2
    for q, hf in zip(b_reqs, host_frames):
        assert np.array_equal(q.escape_iteration, hf), "batched frames differ from single-frame renders"
    bat2.close()
    e2e_batch_value = eb_eff / eb_t / 1e9

    # zoom sequence (zoom.py): a stated subset of the 600 frames at the frames'
    # resolution, EDE, mixed form, one periodic reference orbit shared by every
    # frame (built once, outside the timed frames); accuracy on the committed
    # arbitrary-precision subsets of five 240x136 frames of the sequence
    import zoom

    zsub = list(range(0, zoom.ZOOM_FRAMES, 50)) + [zoom.ZOOM_FRAMES - 1]
    zbe = mbx.create_compute_backend("cuda", local)
    zoom.render_sequence(zbe, [zsub[1]], W, H)  # builds the shared orbit
    zframes = {}
    z_t0 = time.perf_counter()
    for k, q, st in zoom.render_sequence(zbe, zsub, W, H):
        zframes[k] = {"frame_ms": st["total_ms"], "pass_gpu_ms": st["pass_gpu_ms"], "effective_iterations": st["effective_iterations"],
                      "reused_reference": st["reused_reference"], "reruns": st["fp64_reruns"], "maxiter": q.max_iterations}
    z_elapsed = time.perf_counter() - z_t0
    z_acc = {}
    ztp = os.path.join(ROOT, "tests", "golden", "truth_zoom.npz")
    if os.path.exists(ztp):
        zt = np.load(ztp)
        for k, q, st in zoom.render_sequence(zbe, [8, 150, 300, 450, 599], 240, 136):
            idx, tn, tv = zt["idx_%d" % k], zt["N_%d" % k], zt["value_%d" % k]
            ext = (tn > 0) & (q.escape_iteration[idx] == tn)
            z_acc[k] = {"escape_iteration_identical": float(np.mean(q.escape_iteration[idx] == tn)),
                        "max_rel_dDE": float(np.max(np.abs(q.iterations[idx][ext].astype(np.float64) - tv[ext]) / np.abs(tv[ext]), initial=0.0))}
    zbe.close()
    zoom_line = {"frames": len(zsub), "subset": "frames 0, 50, ..., 550, 599 of 600 (half-width 10^(-1000 k/599), maxiter 1e3 -> 5e6 geometric, EDE)",
                 "ms_total": z_elapsed * 1e3, "frame_ms": {str(k): v["frame_ms"] for k, v in zframes.items()},
                 "gpixel_iter_per_s": sum(v["effective_iterations"] for v in zframes.values()) / z_elapsed / 1e9, "unit": UNIT,
                 "shared_orbit": "period-%d nucleus, built once; reused by %d of %d frames (the shallow ones, half-width >= 2e-6, use no reference)"
                                 % (zoom.target()[2], sum(v["reused_reference"] for v in zframes.values()), len(zsub)),
                 "accuracy_vs_truth_240x136": z_acc}

    # batching workload (views.c3_views): all 64 views at 1/8 of their linear
    # sizes (32..512 square, half of them 3x3 adaptive supersampling), one
    # mbx_compute_batch call per step with the references resident: the views'
    # probe and main passes in one CUDA graph, then the supersampling passes
    c3 = views.c3_views(size_div=8)
    c3be = mbx.create_compute_backend("cuda", local)

    def c3_reqs():
        return [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], v["width"], v["height"], v["max_iterations"], sub=v["sub"],
                                   coloring_method=v["coloring_method"], bailout=v["bailout"], precision_bits=v["precision_bits"],
                                   precision_mode=mbx.PRECISION_MIXED, reuse_reference=True) for v in c3]
    for _ in range(2):
        assert c3be.compute_batch(c3_reqs()) == mbx.OK, c3be.last_error()
    c3_t, c3_eff, c3_gpu = 0.0, 0, 0.0
    for _ in range(args.steps):
        rq = c3_reqs()
        t = time.perf_counter()
        assert c3be.compute_batch(rq) == mbx.OK, c3be.last_error()
        c3_t += time.perf_counter() - t
        c3_eff += c3be.last_batch_stats.effective_iterations + sum(s_.effective_iterations for s_ in c3be.last_view_stats)
        c3_gpu += c3be.last_batch_stats.pass_gpu_ms
    c3be.close()
    c3_line = {"views": len(c3), "sample": "all 64 seed-drawn views at 1/8 of their linear sizes (32..512 square; 32 with 3x3 adaptive supersampling), references resident",
               "ms_per_batch": c3_t / args.steps * 1e3, "shared_graph_gpu_ms": c3_gpu / args.steps, "gpixel_iter_per_s": c3_eff / c3_t / 1e9, "unit": UNIT}

    # learned-scheduling workload (views.c4_tiles): 24 seed-drawn 256x256 tiles
    # of the 23040x12960 image (7680x4320 with 3x3 uniform supersampling) at
    # half-width 1e-500 by a period-38045 minibrot's edge, maxiter 2e6, as one
    # mbx_compute_batch per step: natural order, the untrained model (tiles by
    # mean probe cost), and the committed weights trained further on the batch
    c4 = views.c4_tiles(n=24)
    c4be = mbx.create_compute_backend("cuda", local)

    def c4_reqs():
        return [mbx.ComputeRequest(v["center_re"], v["center_im"], v["scale"], v["width"], v["height"], v["max_iterations"], bailout=v["bailout"],
                                   precision_bits=v["precision_bits"], precision_mode=mbx.PRECISION_MIXED, reference_re=v["reference_re"],
                                   reference_im=v["reference_im"], reference_period=v["reference_period"]) for v in c4]

    def c4_time(k):
        t_, eff_, f32_, g_, out_ = 0.0, 0, 0.0, 0.0, None
        for _ in range(k):
            rq = c4_reqs()
            t = time.perf_counter()
            assert c4be.compute_batch(rq) == mbx.OK, c4be.last_error()
            t_ += time.perf_counter() - t
            bs_ = c4be.last_batch_stats
            eff_ += bs_.effective_iterations + sum(s_.effective_iterations for s_ in c4be.last_view_stats)
            f32_ += bs_.fp32_pass_gpu_ms
            g_ += bs_.pass_gpu_ms
            out_ = [r.escape_iteration.copy() for r in rq]
        return {"ms_per_batch": t_ / k * 1e3, "fp32_pass_gpu_ms": f32_ / k, "shared_graph_gpu_ms": g_ / k, "gpixel_iter_per_s": eff_ / t_ / 1e9}, out_

    c4_init = order_train.initial_params()
    c4be.set_batch_scheduling(0)
    c4_time(1)  # the engines' orbits and tables
    c4_nat, c4_o0 = c4_time(args.steps)
    c4be.schedule_params(c4_init)
    c4be.set_batch_scheduling(2)
    c4_time(1)
    c4_un, c4_o1 = c4_time(args.steps)
    order_train.load_weights(c4be)
    c4be.set_batch_scheduling(1)
    c4_time(1)  # trains on this batch's map
    c4be.set_batch_scheduling(2)
    c4_tr, c4_o2 = c4_time(args.steps)
    c4be.close()
    c4_samples = sum(v["width"] * v["height"] for v in c4)
    c4_line = {"tiles": len(c4), "sample": "24 seed-drawn 256x256 tiles (%d samples) of the 23040x12960 image; half-width 1e-500, maxiter 2e6" % c4_samples,
               "natural": c4_nat, "untrained_model": c4_un, "trained_model": c4_tr, "unit": UNIT,
               "identical_outputs": all(np.array_equal(a, b) and np.array_equal(a, c) for a, b, c in zip(c4_o0, c4_o1, c4_o2)),
               "full_image_s_at_trained_rate": c4_tr["ms_per_batch"] / 1e3 * (views.C4_W * views.C4_H) / c4_samples,
               "model": "order_model_params.npz (trained offline by order_train.py on the maps of the 1280x720 1e-30 view and the three benchmark frames), 32 Adam steps on the batch"}

    # plain FP64 GPU form on a sample of the same views, and accuracy vs it
    if args.plain_sample == "full":
        pw, ph = W, H
    else:
        pw, ph = (int(x) for x in args.plain_sample.split("x"))
    plain_eff, plain_t, agree, total, cls_mis = 0, 0.0, 0, 0, 0
    plain_frame_ms = []
    for v in vlist:
        req_e, st_e = render(be, mbx, v, mbx.PRECISION_EXACT, width=pw, height=ph)
        req_e2, st_e2 = render(be, mbx, v, mbx.PRECISION_EXACT, width=pw, height=ph, reuse=True)
        plain_t += st_e2["total_ms"] / 1e3
        plain_eff += st_e2["effective_iterations"]
        plain_frame_ms.append(st_e2["total_ms"] * (W * H) / (pw * ph))
        req_m, _ = render(be, mbx, v, mbx.PRECISION_MIXED, width=pw, height=ph)
        agree += int(np.sum(req_m.escape_iteration == req_e.escape_iteration))
        cls_mis += int(np.sum((req_m.escape_iteration < 0) != (req_e.escape_iteration < 0)))
        total += req_e.escape_iteration.size
    plain_value = plain_eff / plain_t / 1e9

    # roofline: the dominant kernel (the FP32 lane passes, k_lane_pass<float>)
    # on its own steps, BLA applies and CUDA-event time; beside it, every
    # delta pass of the frames (all tiers) over the passes' time
    flops = FLOPS_PER_STEP * tot[1] + FLOPS_PER_BLA * tot[2]
    achieved_all = flops / (tot[4] / 1e3) / 1e12 if tot[4] > 0 else 0.0
    k_ms = sum(pf["fp32_ms"] for pf in per_frame.values())
    k_flops = sum(FLOPS_PER_STEP * pf["fp32_steps"] + FLOPS_PER_BLA * pf["fp32_bla"] for pf in per_frame.values())
    achieved = k_flops / (k_ms / 1e3) / 1e12 if k_ms > 0 else 0.0
    frames = {}
    for v in vlist:
        pf = per_frame[v["label"]]
        sec = pf["gpu_ms"] / 1e3
        frames[v["label"]] = {
            "frame_ms": float(frame_ms[[u["label"] for u in vlist].index(v["label"])] / args.steps),
            "pass_gpu_ms": pf["gpu_ms"] / args.steps,
            "gpixel_iter_per_s": pf["eff"] / sec / 1e9 if sec > 0 else None,
            "executed_steps_per_s": pf["steps"] / sec if sec > 0 else None,
            "bla_applies_per_s": pf["bla"] / sec if sec > 0 else None,
            # device time of the tiers (CUDA events): FP32 lanes, double-float lanes, exact form
            "tier_gpu_ms": {"fp32": pf["fp32_ms"] / args.steps, "double_float": (pf["rerun_ms"] - pf["exact_ms"]) / args.steps,
                            "exact_form": pf["exact_ms"] / args.steps},
            "fp32_pass": {"gpu_ms": pf["fp32_ms"] / args.steps, "steps": pf["fp32_steps"] // args.steps, "bla_applies": pf["fp32_bla"] // args.steps,
                          "tflops": (FLOPS_PER_STEP * pf["fp32_steps"] + FLOPS_PER_BLA * pf["fp32_bla"]) / (pf["fp32_ms"] / 1e3) / 1e12 if pf["fp32_ms"] > 0 else None},
        }
    # accuracy at the configuration: the timed frames' mixed-form outputs on
    # each frame's committed arbitrary-precision truth subset (4096 samples,
    # tests/golden/make_truth.py)
    truth_acc = {}
    for v, o in zip(vlist, outs):
        tp = os.path.join(ROOT, "tests", "golden", "truth_c2_%s.npz" % v["label"])
        if not os.path.exists(tp) or (W, H) != (1920, 1080):
            continue
        z = np.load(tp)
        idx = torch.from_numpy(z["idx"].astype(np.int64)).cuda()
        en = o[1][idx].cpu().numpy()
        mu = o[0][idx].cpu().numpy().astype(np.float64)
        tn, tv = z["N"], z["value"].astype(np.float64)
        ext = (tn > 0) & (en > 0)
        truth_acc[v["label"]] = {"samples": int(idx.numel()), "escape_iteration_identical": float(np.mean(en == tn)), "class_mismatch": int(np.sum((en < 0) != (tn < 0))),
                                 "max_abs_dmu": float(np.max(np.abs(mu[ext] - tv[ext]), initial=0.0))}

    # share of the step's device time per tier (all frames)
    tot_tier = {"fp32": 0.0, "double_float": 0.0, "exact_form": 0.0}
    for f_ in frames.values():
        for k_, x_ in f_["tier_gpu_ms"].items():
            tot_tier[k_] += x_
    s_ = sum(tot_tier.values()) or 1.0
    tier_share = {k_: {"gpu_ms": x_, "share": x_ / s_} for k_, x_ in tot_tier.items()}

    cpu = None
    if rank == 0:
        sw_, sh_ = sw, sh
        cpu_v, cpu_dt, cpu_eff = cpu_reference(vlist, sw_, sh_, threads)
        cpu = {"value": cpu_v, "unit": UNIT, "cores": threads, "kind": "port", "sample": "the three views at %dx%d (same view regions; %.1f s, %.3g pixel-iterations) by the oracle, the CPU restatement of the reference path" % (sw_, sh_, cpu_dt, cpu_eff)}

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 (floatexp; f64 decisions)",
            "data": "synthetic",
            "config": {
                "workload": "1080p deep frames: the precision frames (half-width 1e-300 and 1e-1000 at 1e-(k+5) from the period-14164 nucleus) and a 1e-1000 frame holding a whole period-1331 minibrot; maxiter 1e6, bailout 2^8",
                "frames_per_step": len(vlist),
                "resolution": "%dx%d" % (W, H),
                "l2": "inputs (orbit, BLA table) L2/smem resident by design; outputs 2x 8.3 MB written per frame; no flush",
                "frame_ms": {v["label"]: float(ms / args.steps) for v, ms in zip(vlist, frame_ms)},
                "frames": frames,
                "autotuned": tuning,
                "batched": batched,
                "image_epilogue": epilogue,
                "zoom_sequence": zoom_line,
                "batch_c3": c3_line,
                "learned_order_c4": c4_line,
                "reruns_per_frame": reruns,
            },
            "e2e": {"value": e2e_batch_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": eb_t / 2 * 1e3,
                    "api": "mbx_compute_batch (all frames per call, host buffers, fresh GMP references)",
                    "per_frame_api": {"value": e2e_value, "frame_ms": e2e_t / len(vlist) * 1e3, "api": "mbx_compute, one frame per call"}},
            "plain_fp64": {"value": plain_value, "unit": UNIT, "sample": "%dx%d" % (pw, ph), "frame_ms_scaled_to_1080p": plain_frame_ms},
            "tuned_vs_plain": value / plain_value if plain_value > 0 else None,
            # per frame: plain FP64 frame time over the tuned form's (mixed, one
            # frame per mbx_compute) and over the learned-scheduled batch form's
            "vs_plain_per_frame": {v["label"]: {"mixed": plain_frame_ms[i] / frames[v["label"]]["frame_ms"],
                                                 "mixed_learned": (plain_frame_ms[i] / batched["learned_order"]["frame_ms"][v["label"]]) if v["label"] in batched["learned_order"]["frame_ms"] else None}
                                   for i, v in enumerate(vlist)},
            "accuracy": {"vs_truth": truth_acc,
                         "vs_exact_fp64": {"escape_iteration_identical": agree / total if total else None, "class_mismatch": cls_mis, "samples": total}},
            "roofline": {"bound": "fp32", "kernel": "k_lane_pass<float> (FP32 lane passes: probe + main)", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak if fp32_peak else None, "traffic": None,
                         "algorithmic": "25 flops per executed delta step + 19 per BLA application (mp.cpp:2457-2469, 2558, 2732-2740), over the kernel's CUDA-event time",
                         "all_passes": {"achieved": achieved_all, "frac": achieved_all / fp32_peak if fp32_peak else None, "note": "every delta pass of the frames (FP32, double-float and exact-form tiers) over their GPU time"},
                         "peak_source": "measured in-run FMA issue rate (mbx_measure_fma_peak); MEASURED_PEAKS.json holds only HBM and bf16", "fp64_peak": fp64_peak,
                         "step_time_by_tier": tier_share,
                         "note_largest": "by device time the double-float tier (k_lane_pass<df32>) is the step's largest kernel, on the minibrot frame: latency-bound chains of the longest samples (profiles/k_lane_pass_df32_minibrot1000_1080p_ncu.md), far below any throughput roof; the FP32 lane is reported as the roofline kernel because it carries the step's arithmetic"},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": tot[3],
        }
        print(json.dumps(line))
    for cx in ctxs:
        cx.close()
    be.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
