"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/vfem_oracle.cpp`` with g++ and OpenMP into
``oracle/_build/libvfem_oracle.so``. Only the tests, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py`` load it.

The reference itself cannot be compiled here (its MeshFEM submodule, Eigen,
TBB and CHOLMOD are absent), so there is no ``oracle/_ref`` build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "vfem_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvfem_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
