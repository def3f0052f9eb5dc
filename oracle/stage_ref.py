"""Stages the reference's sources that oracle/Makefile.ref and oracle/ref_gpu/build.py compile into
oracle/_ref/src/, so that a machine without the reference tree can build oracle/_ref/libvfref.so
(its CPU code) and oracle/_ref/libvfref_gpu.so (its per-frame GPU loop) for itself.

Test and baseline infrastructure only: oracle/_ref/ is git-ignored (never committed) and holds
the reference's files unchanged, in the reference's own layout (src/, include/af/, the two
third-party header libraries), next to the library built from them.

    python oracle/stage_ref.py <reference tree>      (or VF_REFERENCE=<tree>)
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEST = os.path.join(HERE, "_ref", "src")
SOURCES = ["src/TSDFVolume.cpp", "src/MarchingCubes.cpp", "src/GraphBuilder.cpp", "src/MotionGraph.cpp", "src/Mesh.cpp",
           "src/CameraCalibration.cpp",
           # the per-frame loop and its CUDA sources, for the reference-GPU baseline (oracle/ref_gpu/build.py)
           "src/VolumeFusion.cu", "src/TSDFIntegration.cu", "src/TSDFWarp.cu", "src/MarchingCubes.cu",
           "src/ComputeCorrespondence.cu", "src/VertexManipulation.cu", "src/MotionOptimization.cu",
           "src/LinearSolver.cu", "src/BilateralFilter.cu", "src/Helper.cu"]
TREES = ["include/af", "third_party/include/eigen-master/Eigen", "third_party/include/nanoflann"]


def stage(ref):
    for rel in SOURCES:
        dst = os.path.join(DEST, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(ref, rel), dst)
    for rel in TREES:
        dst = os.path.join(DEST, rel)
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        shutil.copytree(os.path.join(ref, rel), dst)
    return DEST


def staged():
    return all(os.path.exists(os.path.join(DEST, rel)) for rel in SOURCES + TREES)


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VF_REFERENCE", "")
    if not tree or not os.path.isdir(os.path.join(tree, "src")):
        sys.exit("usage: stage_ref.py <reference tree>")
    print(stage(tree))
