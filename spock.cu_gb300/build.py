"""Build libspock_gb300.so (CUDA for sm_103a + C++ host + C ABI) in-tree with nvcc.

Usage: python spock.cu_gb300/build.py      (or `build()` from Python)
Output: spock.cu_gb300/_build/libspock_gb300.so
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libspock_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "problem.cpp", "capi.cpp", "noalloc.cu", "offline.cu", "mlp.cu", "umma_gemm.cu", "ops_batch.cu"]
# ops_batch.cu is compiled once per batched operator kernel, precision, mode and matrix placement
OPS_VARIANTS = [(k, t, m, g) for k in ("LSTAR", "LOP") for t in ("float", "double") for m in (0, 1, 2) for g in (0, 1)]


def _jobs():
    jobs = [(s, [], s + ".o") for s in SOURCES if s != "ops_batch.cu"]
    for k, t, m, g in OPS_VARIANTS:
        jobs.append(("ops_batch.cu", [f"-DSPOCK_OPS_{k}", f"-DSPOCK_OPS_T={t}", f"-DSPOCK_OPS_MODE={m}",
                                      f"-DSPOCK_OPS_GM={g}"], f"ops_{k.lower()}_{t}_{m}_{g}.o"))
    # the slowest units first
    jobs.sort(key=lambda j: (not j[0].startswith("ops"), j[0] != "engine.cu"))
    return jobs


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(job):
    src, defs, name = job
    obj = os.path.join(OUT, name)
    cmd = [nvcc(), "-c", os.path.join(SRC, src), "-o", obj, "-std=c++17", "-O3", "-lineinfo",
           "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr"] + defs + ARCH
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    subprocess.check_call(cmd)
    return obj


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(SRC, s) for s in SOURCES]
    hdrs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".hpp", ".h"))]
    hdrs.append(os.path.join(HERE, "..", "include", "spock_gb300.h"))
    if os.path.exists(LIB):
        newest = max(os.path.getmtime(f) for f in srcs + hdrs)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    jobs = _jobs()
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), max(2, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(_compile, jobs))
    subprocess.check_call([nvcc(), "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart"])
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
