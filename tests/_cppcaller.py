"""Builds tests/cpp/af_surface_check.cpp, a C++ caller of the af:: surface, with the host g++
against include/ and volumefusion_gb300/libafx.so (static CUDA runtime)."""
import glob
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SOURCE = os.path.join(ROOT, "tests", "cpp", "af_surface_check.cpp")
LIBDIR = os.path.join(ROOT, "volumefusion_gb300")


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(os.path.join(c, "include")):
            return c
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(nvcc)) if nvcc else None


def cuda_libdir(home):
    for d in [os.path.join(home, "lib64")] + sorted(glob.glob(os.path.join(home, "targets", "*", "lib"))):
        if os.path.exists(os.path.join(d, "libcudart_static.a")):
            return d
    return None


def compile_caller(out, eigen_include=None, syntax_only=False):
    """Returns the CompletedProcess of g++ (out: the executable; unused with syntax_only)."""
    gxx = shutil.which("g++")
    home = cuda_home()
    if not gxx or not home:
        return None
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(home, "include")]
    if eigen_include:
        cmd += ["-DAFX_TEST_WITH_EIGEN", "-I", eigen_include]
    if syntax_only:
        return subprocess.run(cmd + ["-fsyntax-only", SOURCE], capture_output=True, text=True)
    libdir = cuda_libdir(home)
    if not libdir:
        return None
    cmd += [SOURCE, "-o", out, "-L", LIBDIR, "-lafx", "-Wl,-rpath," + LIBDIR, "-L", libdir, "-lcudart_static",
            "-ldl", "-lpthread", "-lrt"]
    return subprocess.run(cmd, capture_output=True, text=True)
