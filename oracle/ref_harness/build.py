"""Build recipe for the reference harness (test infrastructure only).

Compiles oracle/ref_harness/ref_harness.cpp (dosecalc-beam kernels),
ref_beamlet_harness.cpp (dosecalc-beamlet kernels) and ref_kernel_harness.cpp
(spectrum + kernel-table build), which include the reference's own sources
from the reference checkout, into oracle/_ref/libccref.so,
libccref_beamlet.so and libccref_kernel.so with the host C++
compiler (kernels executed on the CPU through cuda_cpu_shim.h).  Needs the reference checkout; the library is git-ignored
and is only used to pin the oracle and to regenerate tests/golden.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libccref.so")
LIBS = {"beam": ("ref_harness.cpp", LIB),
        "beamlet": ("ref_beamlet_harness.cpp", os.path.join(OUT, "libccref_beamlet.so")),
        "kernel": ("ref_kernel_harness.cpp", os.path.join(OUT, "libccref_kernel.so"))}
HOW = ("set CCCS_REFERENCE to the reference checkout (the directory that holds CCCS/), "
       "or place the checkout beside this repository as ../reference")


def reference_root():
    """The reference checkout: $CCCS_REFERENCE, else a `reference` directory
    beside this repository; None when neither holds CCCS/dosecalc-beam."""
    env = os.environ.get("CCCS_REFERENCE")
    cands = [env] if env else [os.path.join(os.path.dirname(ORACLE), "..", "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "CCCS", "dosecalc-beam")):
            return os.path.abspath(c)
    return None


REF = reference_root()


def available():
    return REF is not None


def build(verbose=False, which="beam"):
    if not available():
        raise RuntimeError("reference checkout not found: " + HOW)
    os.makedirs(OUT, exist_ok=True)
    srcname, LIB = LIBS[which]
    src = os.path.join(HERE, srcname)
    deps = [src] + [os.path.join(HERE, h) for h in ("cuda_cpu_shim.h", "H5Cpp.h")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-w",
           "-I", HERE,
           "-I", os.path.join(REF, "CCCS"),
           "-I", os.path.join(REF, "CCCS", "include"),
           "-I", os.path.join(REF, "CCCS", "include", "cuda-common"),
           "-I", cuda_inc, src, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    for w in LIBS:
        print(build(verbose=True, which=w))
