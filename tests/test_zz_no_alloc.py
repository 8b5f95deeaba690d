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


@pytest.mark.parametrize("prec", [1, 2])
def test_no_alloc_norm_at_the_scratch_limit(cuda, qcu_lib, prec):
    """nrhs = 64 (the largest the fixed array takes) on a field large
    enough that the reduction launches its full 1024 blocks, so every partial
    of the array is written and read; twice in a row, against the allocating
    entry point and numpy in FP64."""
    torch, Q = cuda, qcu_lib
    fn = no_alloc_fn(Q)
    L, n, nrhs = (8, 8, 8, 16), 3, 64
    vh = S.half_volume(L)
    Q.initGridSize(L, n)
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (410, 411):
        field = packed_field(torch, Q, L, n, nrhs, prec, seed)
        want = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
        Q.norm2_mrhs(want.data_ptr(), field.data_ptr(), prec, nrhs)
        Q.synchronize()
        got = torch.full((nrhs,), float("nan"), dtype=torch.float64, device="cuda")
        assert fn(got.data_ptr(), field.data_ptr(), prec, vh * 4 * n * nrhs, nrhs, stream) == 0, Q.last_error()
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-13)
        count = vh * 4 * n * nrhs * (1 if prec == 1 else 2)  # float64 words the field occupies
        vals = field[:count].view(torch.complex64 if prec == 1 else torch.complex128).cpu().numpy()
        direct = (np.abs(vals.astype(np.complex128).reshape(-1, nrhs)) ** 2).sum(0)
        np.testing.assert_allclose(got.cpu().numpy(), direct, rtol=1e-12)


@pytest.mark.parametrize("nrhs", [65, 128])
def test_no_alloc_rejects_oversized_requests(cuda, qcu_lib, nrhs):
    torch, Q = cuda, qcu_lib
    fn = no_alloc_fn(Q)
    out = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
    field = torch.zeros(nrhs * 12, dtype=torch.complex64, device="cuda")
    rc = fn(out.data_ptr(), field.data_ptr(), 1, 12 * nrhs, nrhs, None)
    assert rc == 11  # QCU_ERR_CAPACITY: more RHS than the fixed scratch holds
    assert "scratch" in Q.last_error()[1]
    Q.clear_error()
