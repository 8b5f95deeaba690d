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


# ---- every BLAS-1 operation through qcuBlasMRHS, against numpy in FP64 ----
CDT = {2: np.complex128, 1: np.complex64}
TOLB = {2: 1e-13, 1: 1e-6}


def _field(torch, n, prec, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    h = ((rng.standard_normal(n) + 1j * rng.standard_normal(n)) * scale).astype(CDT[prec])
    return h, torch.from_numpy(h).cuda()


def _coef(torch, nrhs, seed):
    rng = np.random.default_rng(seed)
    h = rng.standard_normal(nrhs) + 1j * rng.standard_normal(nrhs)
    return h, torch.from_numpy(h).cuda()


def _per_rhs(v, nrhs):
    return np.asarray(v).reshape(-1, nrhs)


def _rel(got, want):
    return float(np.linalg.norm(np.asarray(got) - want) / max(np.linalg.norm(want), 1e-300))


def _r(c, prec):
    """coefficients as the kernel uses them: rounded to FP32 for FP32 arithmetic"""
    return c.astype(np.complex64).astype(np.complex128) if prec == 1 else c


@pytest.fixture
def blas_session(qcu_lib):
    qcu_lib.initGridSize((4, 4, 4, 4), 3)
    return qcu_lib


# (nrhs, complex elements per RHS): one RHS, a count that leaves the last
# vector of a thread half-filled, RHS counts that do not divide a block, and
# a field larger than one wave of blocks
SHAPES = [(1, 4097), (3, 1001), (12, 333), (64, 515), (12, 200003)]


@pytest.mark.parametrize("nrhs,k", SHAPES)
@pytest.mark.parametrize("px,py", [(2, 2), (1, 1), (1, 2), (2, 1)])
def test_blas_axpby_and_norm(cuda, blas_session, nrhs, k, px, py):
    torch, Q = cuda, blas_session
    n = nrhs * k
    xh, x = _field(torch, n, px, 1)
    yh, y = _field(torch, n, py, 2)
    ah, a = _coef(torch, nrhs, 3)
    bh, b = _coef(torch, nrhs, 4)
    low = 1 if 1 in (px, py) else 2
    A = np.tile(_r(ah, low), k)
    B = np.tile(_r(bh, low), k)
    want = A * xh.astype(np.complex128) + B * yh.astype(np.complex128)
    Q.blas_mrhs(Q.BLAS_AXPBY, n, nrhs, x.data_ptr(), px, y.data_ptr(), py, a=a.data_ptr(), b=b.data_ptr())
    Q.synchronize()
    assert _rel(y.cpu().numpy(), want) < TOLB[low]
    if px == py:
        _, y2 = _field(torch, n, py, 2)
        out = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
        Q.blas_mrhs(Q.BLAS_AXPBY_NORM, n, nrhs, x.data_ptr(), px, y2.data_ptr(), py, a=a.data_ptr(), b=b.data_ptr(),
                    out=out.data_ptr())
        Q.synchronize()
        yv = y2.cpu().numpy().astype(np.complex128)
        assert _rel(yv, want) < TOLB[low]
        norms = (np.abs(_per_rhs(yv, nrhs)) ** 2).sum(0)  # of the stored (rounded) result
        np.testing.assert_allclose(out.cpu().numpy(), norms, rtol=TOLB[low])


@pytest.mark.parametrize("nrhs,k", SHAPES)
@pytest.mark.parametrize("prec", [2, 1])
def test_blas_axpbypcz(cuda, blas_session, nrhs, k, prec):
    torch, Q = cuda, blas_session
    n = nrhs * k
    xh, x = _field(torch, n, prec, 5)
    yh, y = _field(torch, n, prec, 6)
    zh, z = _field(torch, n, prec, 7)
    ch = [_coef(torch, nrhs, s) for s in (8, 9, 10)]
    A, B, C = [np.tile(_r(c[0], prec), k) for c in ch]
    want = A * xh + B * yh + C * zh
    Q.blas_mrhs(Q.BLAS_AXPBYPCZ, n, nrhs, x.data_ptr(), prec, y.data_ptr(), prec, z.data_ptr(), prec,
                a=ch[0][1].data_ptr(), b=ch[1][1].data_ptr(), c=ch[2][1].data_ptr())
    Q.synchronize()
    assert _rel(z.cpu().numpy(), want) < TOLB[prec]


@pytest.mark.parametrize("nrhs,k", SHAPES)
@pytest.mark.parametrize("prec", [2, 1])
def test_blas_norms_and_dot(cuda, blas_session, nrhs, k, prec):
    """norm2 with FP64 products (exact for FP32 inputs), norm2 with FP32
    products, and the complex dot sum conj(x) y, per RHS."""
    torch, Q = cuda, blas_session
    n = nrhs * k
    # RHS of very different magnitudes: a per-RHS result cannot borrow from another
    scale = np.tile(10.0 ** np.linspace(-3, 3, nrhs), k)
    xh, x = _field(torch, n, prec, 11, scale)
    yh, y = _field(torch, n, prec, 12)
    xd, yd = xh.astype(np.complex128), yh.astype(np.complex128)
    out = torch.zeros(nrhs, dtype=torch.float64, device="cuda")
    want = (np.abs(_per_rhs(xd, nrhs)) ** 2).sum(0)
    Q.blas_mrhs(Q.BLAS_NORM2, n, nrhs, x.data_ptr(), prec, out=out.data_ptr())
    Q.synchronize()
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-13)
    if prec == 1:
        Q.blas_mrhs(Q.BLAS_NORM2_FP32, n, nrhs, x.data_ptr(), prec, out=out.data_ptr())
        Q.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-6)
    dot = torch.zeros(nrhs, dtype=torch.complex128, device="cuda")
    Q.blas_mrhs(Q.BLAS_CDOT, n, nrhs, x.data_ptr(), prec, y.data_ptr(), prec, out=dot.data_ptr())
    Q.synchronize()
    wantd = (np.conj(_per_rhs(xd, nrhs)) * _per_rhs(yd, nrhs)).sum(0)
    scale_r = np.sqrt(want * (np.abs(_per_rhs(yd, nrhs)) ** 2).sum(0))  # Cauchy-Schwarz bound per RHS
    assert np.all(np.abs(dot.cpu().numpy() - wantd) <= TOLB[prec] * scale_r)


@pytest.mark.parametrize("nrhs,k", SHAPES[:4])
@pytest.mark.parametrize("plo,phi", [(1, 2), (2, 2), (1, 1), (2, 1)])
def test_blas_add_to_and_copy(cuda, blas_session, nrhs, k, plo, phi):
    torch, Q = cuda, blas_session
    n = nrhs * k
    lo_h, lo = _field(torch, n, plo, 13)
    hi_h, hi = _field(torch, n, phi, 14)
    Q.blas_mrhs(Q.BLAS_ADD_TO, n, nrhs, lo.data_ptr(), plo, hi.data_ptr(), phi)
    Q.synchronize()
    want = (lo_h.astype(np.complex128) + hi_h.astype(np.complex128)).astype(CDT[phi])
    assert np.array_equal(hi.cpu().numpy(), want)  # one rounding into the destination
    _, dst = _field(torch, n, phi, 15)
    Q.blas_mrhs(Q.BLAS_COPY, n, nrhs, lo.data_ptr(), plo, dst.data_ptr(), phi)
    Q.synchronize()
    assert np.array_equal(dst.cpu().numpy(), lo_h.astype(CDT[phi]))


def test_blas_rejects_bad_shapes(cuda, blas_session):
    torch, Q = cuda, blas_session
    _, x = _field(torch, 30, 2, 16)
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    for args in ((Q.BLAS_NORM2, 30, 7, x.data_ptr(), 2), (Q.BLAS_NORM2, 0, 1, x.data_ptr(), 2),
                 (Q.BLAS_NORM2, 30, 3, x.data_ptr(), 0), (Q.BLAS_AXPBY, 30, 3, x.data_ptr(), 2),
                 (99, 30, 3, x.data_ptr(), 2)):
        with pytest.raises(Q.QcuError) as e:
            Q.blas_mrhs(*args, out=out.data_ptr())
        assert e.value.code in (2, 3), args
    Q.clear_error()
