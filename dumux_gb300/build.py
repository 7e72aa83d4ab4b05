"""In-tree build of libdumux_gb300.so (sm_103a) with nvcc.

Translation units are compiled in parallel and linked into
dumux_gb300/_lib/libdumux_gb300.so.  assemble.cu and mpfa.cu are compiled without FMA
contraction so the residual and the numeric-difference Jacobian follow the reference's
operation order exactly; host code everywhere is compiled with -ffp-contract=off so
the tabulated coefficients are identical on x86 and Arm hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libdumux_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]

UNITS = {
    "assemble.cu": ["--fmad=false"],
    "linalg.cu": [],
    "wave.cu": [],
    "lanewave.cu": [],
    "api.cu": [],
    "noalloc.cu": [],
    "batch.cu": [],
    "amg.cu": [],
    "mpfa.cu": ["--fmad=false"],
    "stencilwave.cu": [],
    "stencillane.cu": [],
    "linesweep.cu": [],
}


def _nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _sources_newer_than(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)]
    deps.append(os.path.join(HERE, "..", "include", "dumux_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and not _sources_newer_than(LIB):
        return LIB
    nvcc = _nvcc()

    def compile_unit(name):
        obj = os.path.join(OUT_DIR, name + ".o")
        cmd = [nvcc, *ARCH, *COMMON, *UNITS[name], *extra_flags, "-c", os.path.join(SRC, name), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ()))
