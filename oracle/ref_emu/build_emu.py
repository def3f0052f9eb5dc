"""Build oracle/_ref/libvfemu.so: the reference's own CUDA kernel sources executed on the host.

Test infrastructure only (golden vectors for the stages that exist in the reference only as
GPU kernels).  Reads the reference's .cu files where they lie, rewrites only the launch syntax
(``k<<<grid, block[, smem]>>>(args);`` becomes a call into the emulation runtime) and the one
dynamic shared-memory declaration, writes the result under oracle/_ref/emu/ (git-ignored) and
compiles it with g++ against the CUDA stand-in headers in oracle/ref_emu/include.  The kernel
bodies are compiled unchanged.

    python oracle/ref_emu/build_emu.py [REF]
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
GEN = os.path.join(OUT, "emu")
HEADERS = ["Helper.cuh"]
SOURCES = ["Helper.cu", "BilateralFilter.cu", "VertexManipulation.cu", "ComputeCorrespondence.cu",
           "MotionOptimization.cu", "TSDFIntegration.cu", "TSDFWarp.cu", "MarchingCubes.cu"]


def split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{<":
            depth += 1
        elif ch in ")]}>":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def rewrite_launches(src, sync):
    out, pos = [], 0
    while True:
        i = src.find("<<<", pos)
        if i < 0:
            out.append(src[pos:])
            return "".join(out)
        m = re.search(r"([A-Za-z_][A-Za-z0-9_:]*)\s*$", src[pos:i])
        name_start = pos + m.start(1)
        j = src.index(">>>", i)
        cfg = split_top(src[i + 3:j])
        k = src.index("(", j)
        depth, e = 0, k
        while True:
            if src[e] == "(":
                depth += 1
            elif src[e] == ")":
                depth -= 1
                if depth == 0:
                    break
            e += 1
        args = src[k + 1:e]
        semi = src.index(";", e)
        smem = cfg[2] if len(cfg) > 2 else "0"
        fn = "launch_sync" if sync else "launch"
        call = "::af_emu::%s(dim3(%s), dim3(%s), (size_t)(%s), [&]() { %s(%s); });" % (
            fn, cfg[0], cfg[1], smem, src[name_start:i].strip(), args)
        out.append(src[pos:name_start])
        out.append(call)
        pos = semi + 1


def transform(path, header=False):
    src = open(path).read()
    sync = "__syncthreads" in src
    src = re.sub(r"extern\s+__shared__\s+(\w+)\s+(\w+)\s*\[\s*\]\s*;",
                 r"\1* \2 = static_cast<\1*>(::af_emu::dynamic_smem());", src)
    src = rewrite_launches(src, sync)
    return src if header else '#include "af_emu.h"\n' + src


def write_if_changed(dst, text):
    if not os.path.exists(dst) or open(dst).read() != text:
        open(dst, "w").write(text)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VF_REFERENCE", "")
    if not ref:
        sys.exit("usage: build_emu.py <reference tree>  (or set VF_REFERENCE)")
    os.makedirs(os.path.join(GEN, "include", "af"), exist_ok=True)
    for h in HEADERS:
        write_if_changed(os.path.join(GEN, "include", "af", h),
                         transform(os.path.join(ref, "include", "af", h), header=True))
    outs = []
    for s in SOURCES:
        dst = os.path.join(GEN, s.replace(".cu", ".cpp"))
        write_if_changed(dst, transform(os.path.join(ref, "src", s)))
        outs.append(dst)
    inc = ["-I" + os.path.join(GEN, "include"), "-I" + os.path.join(HERE, "include"),
           "-I" + os.path.join(ref, "include"),
           "-I" + os.path.join(ref, "third_party", "include", "eigen-master"),
           "-I" + os.path.join(ORACLE, "ref_shims")]
    lib = os.path.join(OUT, "libvfemu.so")
    deps = outs + [os.path.join(HERE, f) for f in ("af_emu.cpp", "ref_emu_driver.cpp", "build_emu.py")]
    deps += [os.path.join(HERE, "include", f) for f in os.listdir(os.path.join(HERE, "include"))]
    if os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(d) for d in deps if os.path.isfile(d)):
        print(lib)
        return
    cmd = (["g++", "-std=c++17", "-O1", "-fPIC", "-ffp-contract=off", "-w", "-shared", "-include", "af_emu.h"] + inc +
           ["-o", lib, os.path.join(HERE, "af_emu.cpp"),
            os.path.join(HERE, "ref_emu_driver.cpp")] + outs)
    subprocess.run(cmd, check=True)
    print(lib)


if __name__ == "__main__":
    main()
