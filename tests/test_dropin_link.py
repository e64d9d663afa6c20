"""The C++ drop-in layer (include/t9gb_tinker.hpp, libt9gb_tinker.so)
builds with g++, exports the reference's namespace-tinker entry points with
the reference's signatures (the mangled names a Tinker9 build links
against: include/ff/amoeba/induce.h:8-34, empole.h:11-13, epolar.h:10,
emplar.h:14), and a C++ caller links against it.  No GPU calls."""
import importlib
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER_SRC = os.path.join(ROOT, "tests", "dropin", "dropin_driver.cpp")
DRIVER = os.path.join(ROOT, "tests", "dropin", "_build", "dropin_driver")

SIGNATURES = [
    "tinker::induce(float (*) [3], float (*) [3])",
    "tinker::dfield(float (*) [3], float (*) [3])",
    "tinker::ufield(float const (*) [3], float const (*) [3], float (*) [3], float (*) [3])",
    "tinker::diagPrecond(float const (*) [3], float const (*) [3], float (*) [3], float (*) [3])",
    "tinker::sparsePrecondApply(float const (*) [3], float const (*) [3], float (*) [3], float (*) [3])",
    "tinker::mpoleInit(int)",
    "tinker::empole(int)",
    "tinker::epolar(int)",
    "tinker::emplar(int)",
]


def test_tinker_layer_exports_reference_signatures():
    b = importlib.import_module("tinker-gpu_gb300.build")
    b.build()
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", b.LIB_TINKER], capture_output=True, text=True,
                         check=True).stdout
    for sig in SIGNATURES:
        assert sig in out, sig


def test_cxx_caller_links():
    b = importlib.import_module("tinker-gpu_gb300.build")
    exe = b.build_cxx_program(DRIVER_SRC, DRIVER)
    r = subprocess.run([exe, "--link-check"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "linked 4 term entry points" in r.stdout
