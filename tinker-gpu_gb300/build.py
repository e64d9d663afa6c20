"""Build recipe of the CUDA library libt9gb.so (sm_103a only) and of the
C++ drop-in layer libt9gb_tinker.so above it.

Each translation unit under csrc/ compiles in parallel with nvcc, then one
nvcc -shared link produces csrc/_build/libt9gb.so inside the source tree.
t9gb_tinker.cpp (the reference's namespace-tinker entry points, host C++
only) compiles with g++ into csrc/_build/libt9gb_tinker.so, linked against
libt9gb.so and the CUDA runtime.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(CSRC, "_build")
LIB = os.path.join(BUILD, "libt9gb.so")
LIB_TINKER = os.path.join(BUILD, "libt9gb_tinker.so")
INCLUDE = os.path.normpath(os.path.join(HERE, "..", "include"))
SOURCES = ["abi.cu", "nblist.cu", "pair.cu", "pme.cu", "pcg.cu", "energy.cu", "mlp.cu", "learn.cu", "force.cu", "vdw.cu", "valence.cu", "md.cu", "noalloc.cu",
           "dropin.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    deps = [os.path.join(CSRC, src), *headers, os.path.join(HERE, "..", "include", "t9gb.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [_nvcc(), *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def _cuda_home():
    nvcc = _nvcc()
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _cuda_lib_dir():
    home = _cuda_home()
    for d in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        if os.path.exists(os.path.join(home, d, "libcudart.so")):
            return os.path.join(home, d)
    return os.path.join(home, "lib64")


def _newer(out, deps):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps)


def build_tinker_layer():
    """g++ -shared of csrc/t9gb_tinker.cpp into libt9gb_tinker.so (needs libt9gb.so)."""
    src = os.path.join(CSRC, "t9gb_tinker.cpp")
    deps = [src, LIB, os.path.join(INCLUDE, "t9gb.h"), os.path.join(INCLUDE, "t9gb_tinker.hpp")]
    if _newer(LIB_TINKER, deps):
        return LIB_TINKER
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-I", INCLUDE, "-I",
           os.path.join(_cuda_home(), "include"), src, "-o", LIB_TINKER + ".tmp", "-L", BUILD, "-lt9gb", "-L",
           _cuda_lib_dir(), "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + _cuda_lib_dir()]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for t9gb_tinker.cpp:\n{r.stderr}")
    os.replace(LIB_TINKER + ".tmp", LIB_TINKER)
    return LIB_TINKER


def build_cxx_program(src, out):
    """g++ a C++ caller of the drop-in layer (tests use it for their driver)."""
    build()
    deps = [src, LIB_TINKER, LIB, os.path.join(INCLUDE, "t9gb_tinker.hpp")]
    if _newer(out, deps):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, "-I", os.path.join(_cuda_home(), "include"), src,
           "-o", out + ".tmp", "-L", BUILD, "-lt9gb_tinker", "-lt9gb", "-L", _cuda_lib_dir(), "-lcudart",
           "-Wl,-rpath," + BUILD, "-Wl,-rpath," + _cuda_lib_dir()]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {src}:\n{r.stderr}")
    os.replace(out + ".tmp", out)
    return out


def build(force=False, verbose_ptxas=False):
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    objs = [o for o, _ in results]
    logs = "".join(l for _, l in results)
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        build_tinker_layer()
        return LIB, logs
    cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcufft", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    build_tinker_layer()
    return LIB, logs


if __name__ == "__main__":
    import sys

    lib, logs = build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    if logs:
        print(logs)
    print(lib)
