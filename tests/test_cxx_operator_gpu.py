"""GPU parity of the reference-compatible C++ operator interface: a C++
program built against include/qcu_dirac.h (tests/cxx/dirac_caller.cpp)
calls qcu::DiracWilson::Dslash through the Dirac base class,
qcu::instantiateDslash and qcu::WilsonDslash<F, 3, 4>::apply on the
reference's coalesced per-RHS arrays; each result is checked against the
FP64 oracle (periodic boundaries, as the reference's kernel), and an
unsupported operator type is reported through qcuGetLastError() without
ending the process."""
import os
import shutil

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.test_abi import build_cxx_caller
from tests.util import TOL, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def caller(tmp_path_factory, qcu_lib):
    gxx = shutil.which("g++")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if gxx is None:
        pytest.skip("g++ not available")
    return build_cxx_caller(str(tmp_path_factory.mktemp("cxx")), gxx, cuda)


@pytest.mark.parametrize("L,n,nrhs,prec,parity,dagger", [
    ((4, 4, 4, 8), 3, 4, 2, 0, 0), ((4, 4, 4, 8), 3, 4, 1, 1, 1), ((8, 4, 4, 4), 4, 2, 2, 1, 0),
    ((4, 4, 6, 4), 6, 7, 1, 0, 1), ((8, 8, 8, 8), 3, 12, 1, 0, 0)])
def test_reference_operator_routes(cuda, caller, tmp_path, L, n, nrhs, prec, parity, dagger):
    import subprocess
    vh = S.half_volume(L)
    g = S.random_gauge(L, n, seed=600 + n)
    psi = S.random_fermions(L, n, nrhs, seed=601 + nrhs)
    cdt = np.complex128 if prec == 2 else np.complex64
    # the reference's coalesced layouts: gauge [4][2][N*N][Vh], fermion [4N][Vh] per RHS
    g.reshape(4, 2, vh, n * n).transpose(0, 1, 3, 2).astype(cdt).tofile(str(tmp_path / "gauge.bin"))
    psi.reshape(nrhs, vh, 4 * n).transpose(0, 2, 1).astype(cdt).tofile(str(tmp_path / "in.bin"))
    r = subprocess.run([caller, str(tmp_path)] + [str(v) for v in L] + [str(n), str(nrhs), str(prec), str(parity),
                                                                      str(dagger)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    codes = [int(line.split()[1]) for line in r.stdout.splitlines() if line.startswith("errors")]
    routes = ["out_dirac.bin", "out_inst.bin"] + (["out_wd.bin"] if (n, nrhs) == (3, 4) else [])
    assert codes[:len(routes)] == [0] * len(routes), r.stdout + r.stderr
    assert codes[-1] == 3  # QCU_ERR_UNSUPPORTED for DSLASH_CLOVER, and the process went on
    want = O.dslash(psi, g, L, parity, dagger, False)
    for route in routes:
        got = np.fromfile(str(tmp_path / route), dtype=cdt).reshape(nrhs, 4 * n, vh).transpose(0, 2, 1)
        got = got.reshape(nrhs, vh, 4, n).astype(np.complex128)
        assert rel(got, want) < TOL[prec], (route, rel(got, want))
