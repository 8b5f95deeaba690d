"""GPU tests of the BLAS-1 reductions exposed at the C ABI (qcuNorm2MRHS):
per-RHS norms of resident MRHS fields against numpy in FP64."""
import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from tests.util import dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [2, 1])
@pytest.mark.parametrize("nrhs", [1, 3, 12, 64])
def test_norm2_mrhs(cuda, qcu_lib, prec, nrhs):
    torch, Q = cuda, qcu_lib
    L, n = (4, 4, 4, 8), 3
    Q.initGridSize(L, n)
    psi = S.random_fermions(L, n, nrhs, seed=300 + nrhs)
    psi *= np.arange(1, nrhs + 1)[:, None, None, None]  # distinct norms per RHS
    src = [dev(torch, psi[r]) for r in range(nrhs)]
    db, _ = Q.field_bytes(prec, nrhs)
    field = torch.empty(db // 8, dtype=torch.float64, device="cuda")
    Q.pack_fermions(field.data_ptr(), None, [s.data_ptr() for s in src], Q.QCU_SRC_EO_HALF, 0, prec)
    out = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
    Q.norm2_mrhs(out.data_ptr(), field.data_ptr(), prec, nrhs)
    Q.synchronize()
    want = np.array([np.vdot(psi[r], psi[r]).real for r in range(nrhs)])
    if prec == 1:  # the field holds FP32-rounded values
        want = np.array([np.vdot(p, p).real for p in psi.astype(np.complex64).astype(np.complex128)])
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-13)
