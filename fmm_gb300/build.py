"""Builds the CUDA library libfmm_gb300.so in-tree for sm_103a.

Each .cu file under csrc/ is compiled by nvcc in parallel
(-gencode arch=compute_103a,code=sm_103a) and linked into
fmm_gb300/_build/libfmm_gb300.so.  No cmake, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfmm_gb300.so")
SOURCES = ["api.cu", "tree.cu", "near.cu", "near_f32.cu", "expansions.cu", "translate.cu", "m2l.cu", "m2l_gemm.cu", "diag.cu", "noalloc.cu", "selector.cu", "qmmm.cu"]
HEADERS = ["common.cuh", "m2l_basis.cuh", "pair.cuh", "dispatch.cuh", "mlp.cuh", "internal.h", "series_tables.h", os.path.join("..", "..", "include", "fmm_gpu.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-O2"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, verbose):
    s = os.path.join(CSRC, src)
    o = os.path.join(OUT, src.replace(".cu", ".o"))
    if not _stale(o, s):
        return o, ""
    extra = ["-Xptxas", "-v"] if verbose else []
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", s, "-o", o + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-6000:]))
    os.replace(o + ".tmp", o)
    return o, r.stderr


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    if force:
        for f in os.listdir(OUT):
            os.remove(os.path.join(OUT, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [r[0] for r in results]
    if verbose:
        for r in results:
            sys.stderr.write(r[1])
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart", "-lpthread"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
