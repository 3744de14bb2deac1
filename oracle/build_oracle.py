"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/oracle.cpp into oracle/_build/liboracle.so (loaded by the tests
and the benchmark's CPU-baseline leg through ctypes) and oracle/_build/oracle_md
(the run_md_simulation command line).  FP contraction is off so the
neighbour-list predicate evaluates exactly as written; OpenMP gives the
multi-threaded CPU baseline.  No -march flags: the same source builds on x86_64
and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function"]


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    obj = os.path.join(OUT, "oracle.o")
    lib = os.path.join(OUT, "liboracle.so")
    exe = os.path.join(OUT, "oracle_md")
    deps = [src, os.path.join(HERE, "oracle.h"),
            os.path.join(HERE, "..", "pfmds_gb300", "csrc", "fortio.h"),
            os.path.join(HERE, "..", "pfmds_gb300", "csrc", "settings.h"),
            os.path.join(HERE, "oracle_main.cpp")]
    newest = max(os.path.getmtime(d) for d in deps)
    if all(os.path.exists(p) and os.path.getmtime(p) >= newest for p in (lib, exe)):
        return lib
    cmds = [
        ["g++", *FLAGS, "-c", src, "-o", obj],
        ["g++", "-shared", "-fopenmp", obj, "-o", lib],
        ["g++", *FLAGS, os.path.join(HERE, "oracle_main.cpp"), obj, "-o", exe],
    ]
    for c in cmds:
        if verbose:
            print(" ".join(c))
        subprocess.run(c, check=True)
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(os.path.join(OUT, "liboracle.so"))
