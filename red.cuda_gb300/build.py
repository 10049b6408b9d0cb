"""Builds libredgb.so in-tree with nvcc for sm_103a (no cmake).

The translation units compile in parallel; the shared library lands in
red.cuda_gb300/_build/.  A build is skipped when the library is newer than
every source.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libredgb.so")
DRIVER = os.path.join(BUILD, "redgb_run")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
UNITS = ["stage_mixed.cu", "stage_fp64.cu", "stage_exact.cu", "stage_fp32.cu", "kernels.cu", "sim.cu", "noalloc.cu",
         "proposer.cu", "populate.cu"]
# The FP32 gravity of the MIXED and FP32 modes flushes FP32 denormals (|x| < 1.2e-38, far below any
# coordinate difference, mass or acceleration of the path), so rsqrtf is the bare hardware reciprocal
# square root; FP64 arithmetic is not affected by the flag.
UNIT_FLAGS = {"stage_mixed.cu": ["-ftz=true"], "stage_fp32.cu": ["-ftz=true"]}


def nvcc():
    for c in [os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"]:
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def sources():
    return [os.path.join(CSRC, u) for u in UNITS]


def deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        [os.path.join(ROOT, "include", "redgb.h"), os.path.abspath(__file__),
         os.path.join(HERE, "driver", "redgb_run.cpp")]


def up_to_date():
    if not os.path.exists(LIB) or not os.path.exists(DRIVER):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in deps() if os.path.exists(d))


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [cc, "-c"] + ARCH + NVCC_FLAGS + UNIT_FLAGS.get(os.path.basename(src), []) + ["-o", obj, src]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), src))
    failed = []
    for p, src in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join("%s:\n%s" % f for f in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    build_driver(verbose)
    return LIB


def build_driver(verbose=False):
    """red's command-line interface over the library: _build/redgb_run."""
    src = os.path.join(HERE, "driver", "redgb_run.cpp")
    tmp = DRIVER + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), src, "-L" + BUILD, "-lredgb",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    build(force="-f" in sys.argv, verbose=True)
    print(LIB)
