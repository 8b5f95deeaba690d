"""Failure detection, in forms that fault, trap or hang no GPU.

* A device-side bounded wait that runs out: a diagnostic kernel waits, with
  the wait the staged kernels use, on an mbarrier that nothing completes,
  with a short bound; the host gets QCU_ERR_DEVICE_TIMEOUT and the context
  stays usable (a dslash afterwards matches the oracle).
* A solve that cannot converge in max_iter = 1 iterations:
  QCU_ERR_NOT_CONVERGED, with per-RHS flags.
* Sources holding NaN or Inf: QCU_ERR_INVALID_ARGUMENT naming them, while
  the other RHS of the same call are still solved (oracle true residual);
  the same through the server's request status.
* A device allocation the GPU cannot satisfy (a gauge field far larger than
  its memory): QCU_ERR_OUT_OF_MEMORY before anything is read, and the
  library keeps working.
* An injected host allocation failure (QCU_INJECT_FAILURE):
  QCU_ERR_OUT_OF_MEMORY, then normal operation once it is cleared."""
import os

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import TOL, abi_dslash, dev, rel

pytestmark = pytest.mark.gpu

L_SMALL = (4, 4, 4, 8)


def _dslash_still_works(torch, Q):
    g = S.random_gauge(L_SMALL, 3, seed=700)
    psi = S.random_fermions(L_SMALL, 3, 4, seed=701)
    got = abi_dslash(torch, Q, psi, g, L_SMALL, 0, 0, 1, antiperiodic_t=True)
    assert rel(got, O.dslash(psi, g, L_SMALL, 0, 0, True)) < TOL[1]


@pytest.mark.parametrize("limit", [0.002, 0.05])
def test_device_wait_timeout_reported(cuda, qcu_lib, limit):
    Q = qcu_lib
    Q.clear_error()
    assert Q.check_wait_timeout(limit) == 9  # QCU_ERR_DEVICE_TIMEOUT
    assert Q.last_error()[0] == 9
    Q.clear_error()
    assert Q.check_wait_timeout(limit) == 9  # the flag was reset after the report
    Q.clear_error()
    _dslash_still_works(cuda, Q)
    assert Q.check_wait_timeout(0.0) == 2  # a bound outside (0, 1] is refused before any launch
    Q.clear_error()


def _solve_setup(torch, Q, nrhs, seed):
    L, n = L_SMALL, 3
    g = S.random_gauge(L, n, seed=seed)
    b = S.random_fermions(L, n, nrhs, seed=seed + 1, parities=2)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(True)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    return L, g, b, dg


def test_not_converged_reported(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L, g, b, keep = _solve_setup(torch, Q, 3, 710)
    db = [dev(torch, b[r]) for r in range(3)]
    dx = [torch.zeros_like(x) for x in db]
    p = Q.solver_params(kappa=0.12, tol=1e-10, inner_precision=1, max_iter=1)
    with pytest.raises(Q.QcuError) as e:
        Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    assert e.value.code == 7  # QCU_ERR_NOT_CONVERGED
    assert not any(p.converged[r] for r in range(3))
    Q.clear_error()
    p = Q.solver_params(kappa=0.12, tol=1e-10, inner_precision=1, max_iter=5000)
    Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    assert all(p.converged[r] for r in range(3))


@pytest.mark.parametrize("poison", [np.nan, np.inf])
def test_non_finite_source_reported(cuda, qcu_lib, poison):
    torch, Q = cuda, qcu_lib
    nrhs, tol = 3, 1e-10
    L, g, b, keep = _solve_setup(torch, Q, nrhs, 720)
    b[1, 1, 5, 2, 1] = poison
    db = [dev(torch, b[r]) for r in range(nrhs)]
    dx = [torch.zeros_like(x) for x in db]
    p = Q.solver_params(kappa=0.12, tol=tol, inner_precision=1, max_iter=5000)
    with pytest.raises(Q.QcuError) as e:
        Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    assert e.value.code == 2 and "source(s) 1 hold" in str(e.value)  # QCU_ERR_INVALID_ARGUMENT, naming source 1
    assert not p.converged[1]
    for r in (0, 2):  # the other sources of the same call are solved
        assert p.converged[r]
        assert O.true_residual(dx[r].cpu().numpy(), b[r], g, L, 0.12, antiperiodic_t=True) < 2 * tol
    Q.clear_error()


def test_non_finite_source_in_server(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L, n = L_SMALL, 3
    g = S.random_gauge(L, n, seed=730)
    dg = dev(torch, g)
    srv = Q.Server(8 << 30, max_slots=8, inner_precision=1)
    try:
        srv.add_gauge(0, L, n, dg.data_ptr(), antiperiodic_t=True)
        good = S.random_fermions(L, n, 2, seed=731, parities=2)
        bad = good.copy()
        bad[0, 0, 3, 1, 2] = np.nan
        dgood, dbad = [dev(torch, x) for x in good], [dev(torch, x) for x in bad]
        xg, xb = [torch.zeros_like(x) for x in dgood], [torch.zeros_like(x) for x in dbad]
        i_bad = srv.submit(0, 0.12, 1e-10, [x.data_ptr() for x in xb], [x.data_ptr() for x in dbad])
        i_good = srv.submit(0, 0.12, 1e-10, [x.data_ptr() for x in xg], [x.data_ptr() for x in dgood])
        info_bad, info_good = srv.wait(i_bad), srv.wait(i_good)
        assert info_bad.done and info_bad.status == 2
        assert info_good.done and info_good.status == 0
        for r in range(2):
            assert O.true_residual(xg[r].cpu().numpy(), good[r], g, L, 0.12, antiperiodic_t=True) < 2e-10
    finally:
        srv.close()


def test_device_allocation_failure_reported(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L, n = (128, 128, 128, 128), 8
    need = 8 * (128 ** 4 // 2) * n * n * 16  # the FP64 gauge copy: about 1.1 TB
    free, total = torch.cuda.mem_get_info()
    if need < 2 * total:
        pytest.skip("this GPU could hold the field; the failure would not be guaranteed")
    tiny = torch.zeros(16, dtype=torch.float64, device="cuda")  # never read: the allocation fails first
    Q.clear_error()
    Q.initGridSize(L, n)
    with pytest.raises(Q.QcuError) as e:
        Q.loadQcuGauge(tiny.data_ptr())
    assert e.value.code == 10  # QCU_ERR_OUT_OF_MEMORY
    Q.clear_error()
    _dslash_still_works(torch, Q)


def test_host_allocation_failure_injected(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    Q.clear_error()
    os.environ["QCU_INJECT_FAILURE"] = "session"
    try:
        with pytest.raises(Q.QcuError) as e:
            Q.initGridSize(L_SMALL, 3)
        assert e.value.code == 10
    finally:
        del os.environ["QCU_INJECT_FAILURE"]
    Q.clear_error()
    _dslash_still_works(torch, Q)
    L, g, b, keep = _solve_setup(torch, Q, 2, 740)
    db = [dev(torch, b[r]) for r in range(2)]
    dx = [torch.zeros_like(x) for x in db]
    os.environ["QCU_INJECT_FAILURE"] = "solver"
    try:
        with pytest.raises(Q.QcuError) as e:
            Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], Q.solver_params(kappa=0.12, tol=1e-8))
        assert e.value.code == 10
    finally:
        del os.environ["QCU_INJECT_FAILURE"]
    Q.clear_error()
    p = Q.solver_params(kappa=0.12, tol=1e-8)
    Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    assert all(p.converged[r] for r in range(2))
