"""In-tree build of the CUDA engine library ``endtoend_gb300/_lib/libee_cccs.so``
and of the ``dosecalc-beam`` / ``dosecalc-beamlet`` command-line programs on
top of it.

nvcc, one ``-gencode`` for sm_103a, the translation units compiled in
parallel, then linked as a shared library with the C ABI of include/ee_cccs.h.
No torch, no cmake: the result loads with ctypes (or any C FFI).  The
programs (csrc/ee_dosecalc_beam.cpp, csrc/ee_dosecalc_beamlet.cpp) are host
C++ that uses only that ABI.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libee_cccs.so")
SOURCES = ["ee_kernels.cu", "ee_api.cpp", "ee_noalloc.cu", "ee_server.cpp", "ee_beamlet.cu", "ee_anneal.cu", "ee_preprocess.cu", "ee_kernel_tables.cu", "ee_roi.cpp"]
HEADERS = ["ee_internal.h", "ee_device.cuh", os.path.join("..", "..", "include", "ee_cccs.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CLI_SRC = os.path.join(CSRC, "ee_dosecalc_beam.cpp")
CLI = os.path.join(OUT_DIR, "dosecalc-beam")
CLIS = {"dosecalc-beam": CLI_SRC, "dosecalc-beamlet": os.path.join(CSRC, "ee_dosecalc_beamlet.cpp")}


def nvcc_path():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + [os.path.normpath(os.path.join(CSRC, h)) for h in HEADERS]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build_cli(verbose=False, force=False):
    """The dosecalc-beam and dosecalc-beamlet programs (host C++ over the C
    ABI; rpath $ORIGIN).  Returns the dosecalc-beam path."""
    build(verbose=verbose, force=force)
    cxx = shutil.which("g++") or shutil.which("c++")
    for name, src in CLIS.items():
        out = os.path.join(OUT_DIR, name)
        deps = (src, LIB, os.path.join(ROOT, "include", "ee_cccs.h"), os.path.join(CSRC, "ee_contract.h"))
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(p) for p in deps):
            continue
        if not cxx:
            raise RuntimeError("a host C++ compiler is required to build " + name)
        tmp = out + ".tmp"
        cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", tmp, "-L", OUT_DIR,
               "-lee_cccs", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        if subprocess.call(cmd) != 0:
            raise RuntimeError("building " + name + " failed")
        os.replace(tmp, out)
    return CLI


def build(verbose=False, force=False):
    """Compile (if stale) and return the library path."""
    if not force and not _stale():
        return LIB
    nvcc = nvcc_path()
    os.makedirs(OUT_DIR, exist_ok=True)
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(ROOT, "include")]
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [nvcc] + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc] + common + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append(subprocess.Popen(cmd))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc compilation of the CCCS engine failed")
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    if subprocess.call(cmd) != 0:
        raise RuntimeError("linking libee_cccs.so failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="-f" in sys.argv))
    print(build_cli(verbose=True, force="-f" in sys.argv))
