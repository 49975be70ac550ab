"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/mbx_oracle.cpp and oracle/mbx_color.cpp into oracle/lib/libmbx_oracle.so with
-ffp-contract=off (the restated operation order must be the executed order on
every host, x86-64 and aarch64 alike) and, when the reference sources are
present, the reference engine itself into oracle/_ref/ via ref_build/Makefile.
"""
import glob
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "libmbx_oracle.so")
# Where the reference project's sources lie (read-only); override with MBX_REFERENCE_DIR.
REFERENCE = os.environ.get("MBX_REFERENCE_DIR", "/root/reference")


def find_libgmp():
    cands = glob.glob("/usr/lib/*-linux-gnu/libgmp.so.10") + glob.glob("/usr/lib64/libgmp.so.10") + glob.glob("/usr/lib/libgmp.so.10")
    if not cands:
        raise RuntimeError("libgmp.so.10 not found")
    return cands[0]


def build_oracle(force=False):
    srcs = [os.path.join(HERE, "mbx_oracle.cpp"), os.path.join(HERE, "mbx_color.cpp")]
    hdr = os.path.join(HERE, "oracle_gmp.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in srcs + [hdr]):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"] + srcs + ["-o", LIB, find_libgmp()]
    subprocess.check_call(cmd)
    return LIB


def build_reference():
    """Compile the reference engine in place (x86-64 only; needs its sources)."""
    if not os.path.isdir(os.path.join(REFERENCE, "src", "engine")) or platform.machine() not in ("x86_64", "AMD64"):
        return None
    subprocess.check_call(["make", "-s", "REF=" + REFERENCE], cwd=os.path.join(HERE, "ref_build"))
    return os.path.join(HERE, "_ref", "mbx_refdump")


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference())
