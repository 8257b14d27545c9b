"""Build recipe of liboz_gb300.so (in-tree, sm_103a only).

Each CUDA/C++ translation unit is compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a) and linked into
ozaie_gb300/liboz_gb300.so.  No CMake, no Triton, no torch extension machinery.
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liboz_gb300.so")
INCLUDE = os.path.normpath(os.path.join(HERE, "..", "include"))

SOURCES = [
    "oz_gemm_v1.cu",
    "oz_gemm_v2.cu",
    "oz_gemm_v3.cu",
    "oz_gemm_v4.cu",
    "oz_gemm_v5.cu",
    "oz_split.cu",
    "oz_capi.cu",
    "oz_noalloc.cu",
    "oz_plan.cpp",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC", "-I", INCLUDE] + ARCH


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "oz_gb300.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + ["-x", "cu" if src.endswith(".cu") else "c++", "-c", os.path.join(CSRC, src),
                                   "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def build(force=False, verbose=False):
    """Compile every translation unit (in parallel) and link liboz_gb300.so."""
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
