"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``cccs_oracle.c`` twice with gcc into ``oracle/_build``:

* ``liboracle64.so`` -- FP64 restatement of the reference chain (the checker);
* ``liboracle32.so`` -- the same source in FP32 with OpenMP (timed CPU baseline).

Plain C, no architecture flags, so it builds identically on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "cccs_oracle.c")


def _up_to_date(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    outs = []
    procs = []
    for real, name in (("double", "liboracle64.so"), ("float", "liboracle32.so")):
        target = os.path.join(OUT, name)
        outs.append(target)
        if _up_to_date(target, [SRC, __file__]):
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math",
               f"-DORC_REAL={real}", SRC, "-o", target + ".tmp", "-lm"]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), target))
    for p, target in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {target}")
        os.replace(target + ".tmp", target)
    return outs


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
