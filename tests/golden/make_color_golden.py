"""Generates the image-epilogue fixtures (run in the build container).

For each case below the reference's own image tool (cbotx/Mandelbrot-Explorer
src/tools/render.cpp, compiled in place by oracle/ref_build/Makefile into
oracle/_ref/mbx_refrender) renders a BMP, and its raw value buffer is kept:

* ``color_<case>.bmp`` — the reference's BMP, byte for byte;
* ``color_<case>.f32`` — the (width*ss) x (height*ss) float32 values it
  coloured (MANDEL_DUMPRAW), followed, for the normal-map and distance-overlay
  cases, by the second buffer, dumped by oracle/_ref/mbx_refdump for the same
  frame and colouring flags (its value buffer must equal the tool's);
* ``color_cases.json`` — the colouring parameters of each case.

The GPU machine has neither the reference sources nor the x86 tools, so these
files travel with the repository.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
RENDER = os.path.join(ROOT, "oracle", "_ref", "mbx_refrender")
DUMP = os.path.join(ROOT, "oracle", "_ref", "mbx_refdump")

SEAHORSE = ("-0.74364388703715", "0.13182590420533")
# reference coloring flags (mandel_perturbation.h:30-49)
EDE, SAC, NORMAL, TRAP, DEOVL = 2, 8, 16, 32, 64
# colour parameters: mapping 0 log-power / 1 tanh (EDE) / 2 stripe average / 3 trap;
# shading 0 none / 1 relief / 2 normal map / 3 distance overlay
CASES = {
    "plain_ss1": dict(view=SEAHORSE, exp="5", mxit=3000, w=80, h=60, ss=1, env={}, cm=0, mapping=0, shading=0),
    "plain_ss3": dict(view=SEAHORSE, exp="5", mxit=3000, w=64, h=48, ss=3, env={}, cm=0, mapping=0, shading=0),
    "dens45_ss2": dict(view=("-0.7453", "0.1127"), exp="3", mxit=5000, w=64, h=48, ss=2, env={"MANDEL_DENS": "45"}, cm=0, mapping=0, shading=0, density=45.0),
    "relief_ss2": dict(view=("-0.75", "0.1"), exp="2", mxit=1000, w=64, h=48, ss=2,
                       env={"MANDEL_RELIEF": "1", "MANDEL_LIGHT_AZ": "1.1", "MANDEL_RELIEF_STR": "2.5"}, cm=0, mapping=0, shading=1, az=1.1, relief=2.5),
    "ede_ss2": dict(view=SEAHORSE, exp="5", mxit=3000, w=64, h=48, ss=2, env={"MANDEL_EDE": "1"}, cm=EDE, mapping=1, shading=0),
    "deovl_ss3": dict(view=SEAHORSE, exp="5", mxit=3000, w=48, h=36, ss=3, env={"MANDEL_DE_OVERLAY": "1", "MANDEL_DE_K": "0.8"}, cm=DEOVL, mapping=0, shading=3, de_k=0.8),
    "normal_ss2": dict(view=SEAHORSE, exp="5", mxit=3000, w=64, h=48, ss=2, env={"MANDEL_NORMAL": "1", "MANDEL_LIGHT_EL": "0.9"}, cm=NORMAL, mapping=0, shading=2, el=0.9),
    "sac_ss1": dict(view=SEAHORSE, exp="5", mxit=3000, w=64, h=48, ss=1, env={"MANDEL_SAC": "1"}, cm=SAC, mapping=2, shading=0),
    "trap_ss1": dict(view=("-0.75", "0.1"), exp="2", mxit=1000, w=64, h=48, ss=1, env={"MANDEL_TRAP": "1"}, cm=TRAP, mapping=3, shading=0),
}


def deep_cases():
    sys.path.insert(0, os.path.join(ROOT, "mandelbrot-explorer_gb300"))
    import views

    v = views.deep_view(300)
    # half-width 1e-300: the tool takes the scale as a decimal magnitude
    return {"deep300_ss1": dict(view=(v["center_re"], v["center_im"]), exp="2e300", mxit=1000000, w=48, h=27, ss=1, env={}, cm=0, mapping=0, shading=0)}


def scale_digits(arg):
    """The tool's scale argument as the integer digit string it passes to GMP (render.cpp:178-200)."""
    if any(ch in arg for ch in "eE."):
        mant, _, e = arg.partition("e") if "e" in arg else arg.partition("E")
        frac = len(mant.split(".")[1]) if "." in mant else 0
        return mant.replace(".", "") + "0" * (int(e or 0) - frac)
    return "1" + "0" * int(arg)


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle

    if not build_oracle.build_reference() or not os.path.exists(RENDER):
        raise SystemExit("reference sources / x86 toolchain unavailable")
    cases = dict(CASES)
    cases.update(deep_cases())
    meta = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, c in cases.items():
            bmp = os.path.join(tmp, name + ".bmp")
            env = dict(os.environ, MANDEL_DUMPRAW="1", OMP_NUM_THREADS=str(os.cpu_count()), **c["env"])
            cx, cy = c["view"]
            subprocess.check_call([RENDER, bmp, str(c["w"]), str(c["h"]), cx, cy, c["exp"], str(c["mxit"]), str(c["ss"])], env=env, stdout=subprocess.DEVNULL)
            values = np.fromfile(bmp + ".raw", dtype=np.float32)
            parts = [values]
            if c["shading"] in (2, 3):
                dump = os.path.join(tmp, name + ".dump")
                ws, hs = c["w"] * c["ss"], c["h"] * c["ss"]
                denv = dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count()))
                subprocess.check_call([DUMP, cx, cy, scale_digits(c["exp"]), str(ws), str(hs), str(c["mxit"]), "1", str(c["cm"]), dump], env=denv, stdout=subprocess.DEVNULL)
                d = np.fromfile(dump, dtype=np.float32).reshape(2, -1)
                if not np.array_equal(d[0].view(np.uint32), values.view(np.uint32)):
                    raise SystemExit("%s: the dump tool's values differ from the render tool's" % name)
                parts.append(d[1])
            np.concatenate(parts).tofile(os.path.join(HERE, "color_%s.f32" % name))
            with open(bmp, "rb") as f, open(os.path.join(HERE, "color_%s.bmp" % name), "wb") as g:
                g.write(f.read())
            meta[name] = dict(width=c["w"], height=c["h"], ss=c["ss"], mapping=c["mapping"], shading=c["shading"], density=c.get("density", 60.0),
                              light_az=c.get("az", 2.3), light_el=c.get("el", 0.55), relief_strength=c.get("relief", 1.0), de_k=c.get("de_k", 1.5))
            print("wrote", name, "values %d, interior %.2f, max %.1f" % (values.size, float(np.mean(values < 0)), float(values.max())))
    with open(os.path.join(HERE, "color_cases.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main()
