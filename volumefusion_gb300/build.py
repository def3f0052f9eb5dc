"""Build libafx.so (the sm_103a CUDA library) in place with nvcc.

Each translation unit is compiled in parallel with
    -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -fmad=false
(-fmad=false keeps every binary32 product and sum separately rounded, which is what
makes the kernels bit-reproducible against the CPU oracle), then linked with the
static CUDA runtime into volumefusion_gb300/libafx.so.

    python -m volumefusion_gb300.build [--force] [--verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libafx.so")
SOURCES = ["afx_prep.cu", "afx_integrate.cu", "afx_scan.cu", "afx_mc.cu", "afx_graph.cu", "afx_gn.cu",
           "afx_fusion.cu", "afx_serve.cu", "afx_io.cu", "afx_stream.cu", "afx_decode.cu", "afx_undistort.cu", "afx_gn_dense.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
FLAGS = [ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
         "-fno-fast-math", "-Xptxas", "-O3", "--expt-relaxed-constexpr"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps(src):
    deps = [os.path.join(CSRC, src)]
    for f in os.listdir(CSRC):
        if f.endswith((".cuh", ".h", ".inc")):
            deps.append(os.path.join(CSRC, f))
    deps.append(os.path.join(os.path.dirname(HERE), "include", "afx", "afx.h"))
    return deps


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, _deps(src)):
            cmd = [cc] + FLAGS + list(extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [cc, ARCH, "-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(LIB)
