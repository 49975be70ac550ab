"""Build recipe for the GB300 renderer library (in-tree, no setuptools).

Compiles the CUDA passes for sm_103a with nvcc and the host engine with g++,
then links mandelbrot-explorer_gb300/lib/libmbx_gb300.so. The exact-form
kernels and all host arithmetic are compiled without FMA contraction: the
reference's operation order is part of the result. Runs in about a minute;
translation units compile in parallel.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libmbx_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def libgmp():
    c = glob.glob("/usr/lib/*-linux-gnu/libgmp.so.10") + glob.glob("/usr/lib64/libgmp.so.10")
    if not c:
        raise RuntimeError("libgmp.so.10 not found")
    return c[0]


def units():
    common_nv = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr", "-Xptxas", "-v"]
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp", "-I" + os.path.join(CUDA, "include")]
    return [
        ("kernels_exact.o", [NVCC] + common_nv + ["-fmad=false", "-c", os.path.join(SRC, "kernels_exact.cu")]),
        ("kernels_mixed.o", [NVCC] + common_nv + ["-fmad=true", "-c", os.path.join(SRC, "kernels_mixed.cu")]),
        ("noalloc.o", [NVCC] + common_nv + ["-fmad=false", "-c", os.path.join(SRC, "noalloc.cu")]),
        ("order_model.o", [NVCC] + common_nv + ["-fmad=true", "-c", os.path.join(SRC, "order_model.cu")]),
        ("color.o", [NVCC] + common_nv + ["-fmad=false", "-c", os.path.join(SRC, "color.cu")]),
        ("engine.o", cxx + ["-c", os.path.join(SRC, "engine.cpp")]),
        ("capi.o", cxx + ["-c", os.path.join(SRC, "capi.cpp")]),
        ("batch.o", cxx + ["-c", os.path.join(SRC, "batch.cpp")]),
        ("parmul.o", cxx + ["-c", os.path.join(SRC, "parmul.cpp")]),
    ]


def sources():
    return glob.glob(os.path.join(SRC, "*")) + [os.path.join(HERE, "..", "include", "mbx_gb300.h"), __file__]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    procs = []
    for obj, cmd in units():
        path = os.path.join(OBJ, obj)
        procs.append((obj, subprocess.Popen(cmd + ["-o", path], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    logs = []
    failed = False
    for obj, p in procs:
        out, _ = p.communicate()
        logs.append((obj, out))
        if p.returncode != 0:
            failed = True
            sys.stderr.write("=== %s failed ===\n%s\n" % (obj, out))
    if failed:
        raise RuntimeError("build failed")
    with open(os.path.join(OUT, "ptxas.log"), "w") as f:
        for obj, out in logs:
            f.write("=== %s\n%s\n" % (obj, out))
    objs = [os.path.join(OBJ, o) for o, _ in units()]
    link = ["g++", "-shared", "-o", LIB] + objs + ["-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64"), libgmp(), "-fopenmp"]
    subprocess.check_call(link)
    if verbose:
        for obj, out in logs:
            print("=== " + obj)
            print(out)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
