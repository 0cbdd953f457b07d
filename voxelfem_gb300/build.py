"""Build the CUDA library ``libvfem.so`` in-tree for sm_103a.

Each translation unit of ``csrc/`` is compiled by nvcc in parallel
(``-gencode arch=compute_103a,code=sm_103a``), then linked into
``voxelfem_gb300/_lib/libvfem.so``. No torch headers are involved: the
library's boundary is the plain C ABI of ``include/vfem.h``.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OBJ_DIR = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "libvfem.so")

SOURCES = ["k_fine.cu", "k_coarse.cu", "k_tail.cu", "k_linalg.cu", "k_topopt.cu", "vfem_element.cpp", "vfem_engine.cpp",
           "vfem_lbl.cpp", "k_q2.cu", "vfem_q2.cpp", "k_tc.cu", "k_lbl.cu", "k_mma.cu", "vfem_mma.cpp", "k_filters.cu", "k_2d.cu", "vfem_2d.cpp", "vfem_capi.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps_mtime():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(ROOT, "include", "vfem.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src, extra):
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + extra + ["-I", CSRC, "-I", os.path.join(ROOT, "include"), "-c",
                                                    os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), res.stdout + res.stderr))
    return obj, res.stderr


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    """Compile (if stale) and return the path of libvfem.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = []
    if "--ptxas-v" in sys.argv:
        extra = ["-Xptxas", "-v"]
    print(build(force="--force" in sys.argv or bool(extra), verbose=bool(extra), extra=extra))
