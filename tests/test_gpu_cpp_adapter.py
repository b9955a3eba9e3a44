"""The C++ drop-in (include/amrs_cns.hpp) used from C++: compute_rhs and
advance through the CNS-like class give the oracle's bits, for the domain as
one box and as a level of 27 uneven boxes (ghosts from neighbours), with
and without a body-force source."""
import os
import subprocess

import numpy as np
import pytest
import torch

from amrsolver_gb300 import build as B
from amrsolver_gb300 import problems as P

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("fx", [0.0, 1.75])
@pytest.mark.parametrize("mode", ["advance", "run"])
@pytest.mark.parametrize("m", [1, 3])
def test_cpp_adapter_bitexact(orc, tmp_path, m, mode, fx):
    assert torch.cuda.is_available()
    lib = B.build()
    exe = str(tmp_path / "cns_adapter")
    subprocess.check_call(["nvcc", "-std=c++17", "-O2", "-o", exe, os.path.join(ROOT, "tests/cpp/cns_adapter_main.cpp"),
                           "-I" + os.path.join(ROOT, "include"), "-L" + os.path.dirname(lib), "-lamrs_gb300",
                           "-Xlinker", "-rpath=" + os.path.dirname(lib)])
    n, nsteps, dt, mu = 16, 3, 1e-2, 1.0 / 1600.0
    U, dx = P.tgv(n)
    fin = tmp_path / "in.bin"
    U.tofile(fin)
    subprocess.check_call([exe, str(fin), str(tmp_path / "rhs.bin"), str(tmp_path / "state.bin"), str(n),
                           str(nsteps), repr(dt), repr(mu), str(m), mode, repr(fx)])
    R = np.fromfile(tmp_path / "rhs.bin").reshape(5, n, n, n)
    S = np.fromfile(tmp_path / "state.bin").reshape(5, n, n, n)
    cl = P.Closures.nondimensional(mu)
    sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1, rhs_source=1 if fx else 0, body_force=(fx, 0.0, 0.0))
    dxinv = [1.0 / h for h in dx]
    Ug = U.copy()
    orc.fill_halo(Ug, (-1, -1, -1), (-1, -1, -1))
    np.testing.assert_array_equal(R, orc.rhs(sc, cl, Ug, dxinv))
    ref = U
    for _ in range(nsteps):
        ref = orc.advance(sc, cl, ref, dxinv, (-1, -1, -1), (-1, -1, -1), dt)
    np.testing.assert_array_equal(S, P.valid(ref))
