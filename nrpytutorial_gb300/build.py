"""Builds libnrgpu.so (the CUDA C-ABI library) in-tree for sm_103a.

Every csrc/*.cu translation unit is compiled by its own nvcc process (in
parallel), then linked into nrpytutorial_gb300/libnrgpu.so.  Objects go to
nrpytutorial_gb300/_build/.  Rebuilds only what changed (by mtime against
the sources and headers).
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnrgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I" + INCLUDE,
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; libnrgpu.so cannot be built")


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max(os.path.getmtime(h) for h in hs) if hs else 0.0


def build(verbose=False, ptxas_verbose=False, jobs=None):
    """Compiles what changed.  $NRGPU_DEFINES (e.g. "-DNRGPU_STAGED_NBUF=3")
    adds preprocessor settings of the kernels' tunables; a change of them
    rebuilds everything."""
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    defines = [d for d in os.environ.get("NRGPU_DEFINES", "").split() if d.startswith("-D")]
    stamp = os.path.join(BUILD, "defines.txt")
    old = open(stamp).read() if os.path.exists(stamp) else ""
    if old != " ".join(defines):
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
        with open(stamp, "w") as f:
            f.write(" ".join(defines))
    hdr_t = _newest_header()
    nv = nvcc()
    extra = (["-Xptxas", "-v"] if ptxas_verbose else []) + defines

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if (not ptxas_verbose and os.path.exists(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_t)):
            return obj, ""
        cmd = [nv] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        return obj, r.stderr

    jobs = jobs or max(2, os.cpu_count() or 2)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(compile_one, sources))
    objs = [o for o, _ in results]
    if verbose or ptxas_verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    newest_obj = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest_obj:
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


if __name__ == "__main__":
    import time
    t = time.time()
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
    print("built in %.1f s" % (time.time() - t))
