"""Generates the parity fixtures in this directory (run in the build container).

* ``ref_<case>.f32`` — the reference engine itself (cbotx/Mandelbrot-Explorer
  src/engine/mandel_perturbation.cpp, compiled in place by
  oracle/ref_build/Makefile into oracle/_ref/mbx_refdump) rendering each case
  of cases.json with MANDEL_COARSE=0 and MANDEL_BAILOUT set to the case's
  bailout. Raw little-endian float32, the reference's buffer layout, followed
  by the DE-overlay buffer when the case sets DE_OVERLAY.
* ``ref_julia_<case>.f32`` — the same engine's Mandel::ComputeJulia for each
  case of julia_cases.json (the dump tool's --julia option).
* ``truth_<name>.f32`` — byte copies of the reference's own golden files
  (tests/golden/*.f32 there: arbitrary-precision ground truth, not engine
  output) for the cases its verify harness checks against them.

The GPU machine has neither the reference sources nor the x86 dump tool, so these
files travel with the repository.
"""
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# The reference project's sources (read-only); override with MBX_REFERENCE_DIR.
REF = os.environ.get("MBX_REFERENCE_DIR", "/root/reference")
DUMP = os.path.join(ROOT, "oracle", "_ref", "mbx_refdump")
TRUTH = {
    "point31": "point_7e31.f32",
    "slowpoint": "slowpoint_7e8.f32",
    "minibrot875": "minibrot875.f32",
    "extref875": "minibrot875_extref.f32",
    "gui875": "minibrot875_gui_ss5.f32",
}


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle

    if not build_oracle.build_reference():
        raise SystemExit("reference sources / x86 toolchain unavailable")
    cases = json.load(open(os.path.join(HERE, "cases.json")))
    only = sys.argv[sys.argv.index("--cases") + 1].split(",") if "--cases" in sys.argv else None
    for name, c in cases.items():
        if only is not None and name not in only:
            continue
        env = dict(os.environ, MANDEL_BAILOUT=repr(float(c["bailout"])), MANDEL_COARSE="0", OMP_NUM_THREADS=str(os.cpu_count()))
        out = os.path.join(HERE, "ref_%s.f32" % name)
        cmd = [DUMP, c["center_re"], c["center_im"], c["scale"], str(c["width"]), str(c["height"]), str(c["max_iterations"]), str(c["sub"]), str(c["coloring_method"]), out]
        subprocess.check_call(cmd, env=env, stdout=subprocess.DEVNULL)
        print("wrote", out)
    if only is not None:
        return
    jcases = json.load(open(os.path.join(HERE, "julia_cases.json")))
    for name, c in jcases.items():
        env = dict(os.environ, MANDEL_BAILOUT=repr(float(c["bailout"])), OMP_NUM_THREADS=str(os.cpu_count()))
        out = os.path.join(HERE, "ref_julia_%s.f32" % name)
        cmd = [DUMP, c["center_re"], c["center_im"], c["scale"], str(c["width"]), str(c["height"]), str(c["max_iterations"]), "1", str(c["coloring_method"]), out]
        if c.get("full_height"):
            cmd += [str(c["full_height"]), str(c["row_base"])]
        cmd += ["--julia", c["fixed_c_re"], c["fixed_c_im"]]
        subprocess.check_call(cmd, env=env, stdout=subprocess.DEVNULL)
        print("wrote", out)
    for name, fn in TRUTH.items():
        shutil.copyfile(os.path.join(REF, "tests", "golden", fn), os.path.join(HERE, "truth_%s.f32" % name))
        print("copied", fn)


if __name__ == "__main__":
    main()
