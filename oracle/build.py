"""Build recipe for the CPU oracle library (test infrastructure only).

`build_oracle()` compiles oracle/cns_oracle.cpp with g++ into
oracle/_build/liboracle.so.  `build_ref(root)` runs oracle/build_ref.sh, which
compiles the reference's own kernel sources from the reference tree `root`
(or $AMRS_REFERENCE_ROOT) into oracle/_ref/libcnsref_*.so; with no tree
named, or none there, it does nothing.
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


def build_ref(refroot=None):
    """Compile the reference sources of the tree `refroot` (default: the
    AMRS_REFERENCE_ROOT environment variable) into oracle/_ref; skipped when
    no tree is named or the named one lacks src/rhs."""
    refroot = refroot or os.environ.get("AMRS_REFERENCE_ROOT")
    if not refroot or not os.path.isdir(os.path.join(refroot, "src", "rhs")):
        return None
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), refroot])
    return REF_LIB


if __name__ == "__main__":
    import sys
    print(build_oracle(force=True))
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None))
