"""Build libhbem.so (the GB300 CUDA library behind include/hbem.h) in-tree.

nvcc, one -gencode for sm_103a, the translation units compiled in parallel and
linked into helmholtzbem_gb300/_lib/libhbem.so.  No cmake, no torch extension:
the library is plain C ABI.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libhbem.so")
SOURCES = ["assemble.cu", "solop.cu", "dense.cu", "lu.cu", "tc_gemm.cu", "rsvd.cu", "arnoldi.cu", "capi.cu", "roots.cu",
           "scatterer.cpp", "fields.cu", "mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code: no floating-point contraction, so that x86-64 and aarch64 hosts (where
# the compiler would otherwise fuse a*b+c into FMAs) give bit-identical results.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xcompiler", "-Wall", "-Xcompiler", "-ffp-contract=off", "-Wno-deprecated-gpu-targets"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "hbem.h"))
    deps.append(os.path.abspath(__file__))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = []
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT_DIR, os.path.splitext(s)[0] + ".o")
        objs.append(obj)
        if _stale(obj, src) or ptxas_info:
            cmd = [nvcc()] + ARCH + FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", src, "-o", obj]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, res):
        if verbose or r.returncode != 0 or ptxas_info:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
