"""qcuNorm2MRHSNoAlloc: the per-RHS norm for callers that cannot allocate
device memory (host callbacks, graph nodes, real-time loops, processes whose
device memory a pool already owns).  Its block partial sums live in a fixed
512 KiB device array inside libqcu.so instead of the session workspace.

Called through the C ABI and checked against the allocating entry point
(qcuNorm2MRHS) on two calls in a row: different precision, RHS count and data,
so stale scratch contents from the first call would show up in the second.
Collected last so that a run stopping at its first failure has already run
every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from tests.util import dev

pytestmark = pytest.mark.gpu


def no_alloc_fn(Q):
    fn = Q.lib().qcuNorm2MRHSNoAlloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def packed_field(torch, Q, L, n, nrhs, prec, seed):
    psi = S.random_fermions(L, n, nrhs, seed=seed)
    psi *= np.linspace(0.5, 3.0, nrhs)[:, None, None, None]
    src = [dev(torch, psi[r]) for r in range(nrhs)]
    db, _ = Q.field_bytes(prec, nrhs)
    field = torch.empty(db // 8, dtype=torch.float64, device="cuda")
    Q.pack_fermions(field.data_ptr(), None, [s.data_ptr() for s in src], Q.QCU_SRC_EO_HALF, 0, prec)
    Q.synchronize()
    return field


def test_no_alloc_norm_matches_allocating_entry_point(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    fn = no_alloc_fn(Q)
    L, n = (4, 4, 4, 8), 3
    vh = S.half_volume(L)
    Q.initGridSize(L, n)
    stream = torch.cuda.current_stream().cuda_stream
    for prec, nrhs, seed in [(1, 12, 400), (2, 5, 401)]:
        field = packed_field(torch, Q, L, n, nrhs, prec, seed)
        want = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
        Q.norm2_mrhs(want.data_ptr(), field.data_ptr(), prec, nrhs)
        Q.synchronize()
        got = torch.full((nrhs,), float("nan"), dtype=torch.float64, device="cuda")
        rc = fn(got.data_ptr(), field.data_ptr(), prec, vh * 4 * n * nrhs, nrhs, stream)
        assert rc == 0, Q.last_error()
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-13)


def test_no_alloc_rejects_oversized_requests(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    fn = no_alloc_fn(Q)
    out = torch.zeros(128, dtype=torch.float64, device="cuda")
    field = torch.zeros(128 * 12, dtype=torch.complex64, device="cuda")
    rc = fn(out.data_ptr(), field.data_ptr(), 1, 12 * 128, 128, None)
    assert rc == 11  # QCU_ERR_CAPACITY: more RHS than the fixed scratch holds
    assert "scratch" in Q.last_error()[1]
    Q.clear_error()
