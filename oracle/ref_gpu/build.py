"""Builds oracle/_ref/libvfref_gpu.so: the reference's own fusion loop (af::runVolumeFusion) and the
CUDA and CPU sources it calls, compiled unchanged for sm_103a, plus oracle/ref_gpu/driver.cu.

Baseline infrastructure only (the benchmark's reference-GPU line); output into the git-ignored
oracle/_ref/.  Sources come from the reference tree given as the argument (or VF_REFERENCE), else
from the copy oracle/stage_ref.py staged in oracle/_ref/src/.  Flags follow the reference's
CMakeLists.txt (--expt-relaxed-constexpr, its definitions), with -O3 for host and device and the
architecture of this GPU; shims/cccl_compat.h is pre-included into the CUDA sources (CUDA 13's
thrust comparator lookup, see there).

    python oracle/ref_gpu/build.py [<reference tree>]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT_DIR, "libvfref_gpu.so")
CU = ["VolumeFusion.cu", "TSDFIntegration.cu", "TSDFWarp.cu", "MarchingCubes.cu", "ComputeCorrespondence.cu",
      "VertexManipulation.cu", "MotionOptimization.cu", "LinearSolver.cu", "BilateralFilter.cu", "Helper.cu"]
CPP = ["GraphBuilder.cpp", "MotionGraph.cpp", "Mesh.cpp"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
COMPAT = os.path.join(HERE, "shims", "cccl_compat.h")
DEFS = ["-D_MWAITXINTRIN_H_INCLUDED", "-D_FORCE_INLINES", "-D__STRICT_ANSI__", "-DVOLUMEFUSION_SOURCE_DIR=."]


def tree(arg=None):
    for t in (arg, os.environ.get("VF_REFERENCE"), os.path.join(ORACLE, "_ref", "src")):
        if t and os.path.isfile(os.path.join(t, "src", "VolumeFusion.cu")):
            return t
    return None


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def build(ref=None, verbose=False):
    ref = tree(ref)
    if ref is None:
        raise RuntimeError("no reference sources (give the tree or stage them with oracle/stage_ref.py)")
    work = os.path.join(OUT_DIR, "gpu_build")
    os.makedirs(work, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "shims"), "-I", os.path.join(ORACLE, "ref_shims"), "-I",
           os.path.join(ref, "include"), "-I", os.path.join(ref, "third_party", "include", "eigen-master"), "-I",
           os.path.join(ref, "third_party", "include", "nanoflann")]
    cc = nvcc()
    jobs = []
    objs = []
    for f in CU:
        o = os.path.join(work, f + ".o")
        objs.append(o)
        jobs.append([cc, ARCH, "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-O3", "-w"]
                    + DEFS + inc + ["-include", COMPAT, "-c", os.path.join(ref, "src", f), "-o", o])
    o = os.path.join(work, "driver.o")
    objs.append(o)
    jobs.append([cc, ARCH, "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-O3", "-w"] + DEFS
                + inc + ["-c", os.path.join(HERE, "driver.cu"), "-o", o])
    for f in CPP:
        o = os.path.join(work, f + ".o")
        objs.append(o)
        jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-w"] + DEFS + inc + ["-c", os.path.join(ref, "src", f),
                                                                              "-o", o])

    def run(cmd):
        t0 = time.time()
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r, time.time() - t0

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for cmd, r, dt in ex.map(run, jobs):
            if verbose:
                print("%6.1fs %s" % (dt, os.path.basename(cmd[-3])), flush=True)
            if r.returncode != 0:
                raise RuntimeError("compile failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr[-4000:]))
    r = subprocess.run([cc, ARCH, "-shared", "-o", LIB] + objs + ["-lcusolver", "-lcublas"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr[-4000:]))
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True))
