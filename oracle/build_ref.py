"""Build recipe of the reference-code harness oracle/_ref/libt9ref.so.

TEST INFRASTRUCTURE ONLY.  Compiles oracle/ref_harness.cpp with g++ against
the Tinker9 headers where they lie in the reference checkout (read-only;
nothing is copied), in double precision, with the reference's own build
macros: TINKER_DOUBLE_PRECISION selects real = double
(include/ff/precision.h:71-76) and TINKER9_DIR the checkout
(include/tool/macro.h:120-125), and include/syntax/acc supplies the host
(non-CUDA) forms of its vector types and routine qualifiers.  The
header-only pair, damping, frame and
B-spline routines compile without the reference's CMake build, its Fortran
Tinker library or FFTW.  Output goes to oracle/_ref/ only; the checkout's
location comes from the T9GB_REFERENCE environment variable (default: the
container's checkout path).  Where the checkout is absent (the GPU host)
build() returns None and the tests that use the harness skip.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libt9ref.so")
SRC = os.path.join(HERE, "ref_harness.cpp")
DEFAULT_CHECKOUT = "/root/reference"


def checkout():
    path = os.environ.get("T9GB_REFERENCE", DEFAULT_CHECKOUT)
    return path if os.path.isfile(os.path.join(path, "include", "seq", "pair_field.h")) else None


def build(force=False):
    """Returns the path of libt9ref.so, or None without the reference checkout."""
    ref = checkout()
    if ref is None:
        return LIB if os.path.exists(LIB) else None
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-DTINKER_DOUBLE_PRECISION", f"-DTINKER9_DIR={ref}",
           "-I", os.path.join(ref, "include"), "-I", os.path.join(ref, "include", "syntax", "acc"), SRC, "-o",
           LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
