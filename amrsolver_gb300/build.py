"""Build recipe of the CUDA library (sm_103a only).

Compiles amrsolver_gb300/csrc/*.cu with nvcc in parallel and links
amrsolver_gb300/_lib/libamrs_gb300.so in the source tree.  The forward
translation units are built with -fmad=false: the kernels keep the
reference's floating-point operation order, and without contraction their
results are bit-identical to the reference's CPU build.  The reverse-mode
units (adjoint*.cu) have no bit-exact counterpart (their bar is agreement
with forward-mode derivatives to ~1e-11 and with finite differences), so
they let the compiler contract a*b + c into fused multiply-adds: on this
FP64-bound path that removes a large share of their FP64 instructions.
"""
import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libamrs_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"] + ARCH


def _fmad(src):
    """-fmad=false for the forward kernels, contraction for the reverse mode."""
    return ["-fmad=true"] if os.path.basename(src).startswith("adjoint") else ["-fmad=false"]


def _sources():
    return sorted(glob.glob(os.path.join(SRC, "*.cu")))


def _deps():
    return sorted(glob.glob(os.path.join(SRC, "*.cu")) + glob.glob(os.path.join(SRC, "*.cuh"))
                  + glob.glob(os.path.join(SRC, "*.h")) + glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    objs = []
    cmds = []
    for s in _sources():
        o = os.path.join(OUT, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        cmds.append([NVCC] + FLAGS + _fmad(s) + list(extra) + ["-c", s, "-o", o])

    def run(c):
        r = subprocess.run(c, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(c), r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(cmds))) as ex:
        for err in ex.map(run, cmds):
            if verbose and err:
                print(err)
    tmp = LIB + ".tmp%d" % os.getpid()
    r = subprocess.run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
