"""Build recipe for the CPU oracle library (test infrastructure only).

`build_oracle()` compiles oracle/cns_oracle.cpp with g++ into
oracle/_build/liboracle.so.  `build_ref()` runs oracle/build_ref.sh, which
compiles the reference's own kernel sources (when the reference tree is
present on this machine) into oracle/_ref/libcnsref.so.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libcnsref_const.so")

CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]


def build_oracle(force=False):
    src = os.path.join(HERE, "cns_oracle.cpp")
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(src)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++"] + CXXFLAGS + ["-o", tmp, src])
    os.replace(tmp, LIB)
    return LIB


def build_ref(refroot="/root/reference"):
    """Compile the reference sources into oracle/_ref (skipped when absent)."""
    if not os.path.isdir(os.path.join(refroot, "src", "rhs")):
        return None
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), refroot])
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref())
