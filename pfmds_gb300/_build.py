"""In-tree build of the CUDA library and the run_md_simulation executable.

Compiles pfmds_gb300/csrc/*.cu for sm_103a only (one -gencode, -lineinfo) in
parallel, links pfmds_gb300/_build/libpfmd.so and the drop-in executable
pfmds_gb300/_build/run_md_simulation (rpath $ORIGIN).  Rebuilds only what changed.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
CU_SOURCES = ["nlist.cu", "forces_pair.cu", "forces_rjl.cu", "forces_tb.cu", "forces_rebo.cu", "forces_cos.cu", "integrate.cu", "noalloc.cu", "batch.cu", "learned.cu", "learned_tc.cu",
              "engine.cu", "cli.cu", "fit.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
EXECUTABLES = [("run_md_simulation", "pfmd_run_md_simulation"), ("run_gr_analysis", "pfmd_run_gr_analysis"),
               ("run_gr_moire_fitting", "pfmd_run_gr_moire_fitting")]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pfmds_gb300")
    return p


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "pfmd.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose=False, jobs=None):
    """Builds libpfmd.so and run_md_simulation; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    headers = _headers()
    objs = []
    todo = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            todo.append([nvcc(), *NVCC_FLAGS, "-c", s, "-o", o])
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), todo))
    lib = os.path.join(OUT, "libpfmd.so")
    if _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", lib, *objs], verbose)
    # the drop-in executables: each main() calls its pfmd_run_* entry point
    for name, entry in EXECUTABLES:
        exe = os.path.join(OUT, name)
        main = os.path.join(OUT, name + "_main.cpp")
        text = ('#include "pfmd.h"\n'
                f"int main(int argc, char** argv) {{ return {entry}(argc, argv); }}\n")
        if not os.path.exists(main) or open(main).read() != text:
            with open(main, "w") as f:
                f.write(text)
        if _stale(exe, [lib, main]):
            _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, main, "-o", exe, "-L" + OUT, "-lpfmd",
                  "-Wl,-rpath,$ORIGIN"], verbose)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
