"""Wilson-clover operator M = A - kappa D.  The reference defines only the
clover storage (include/basic_data/qcu_point.cuh:98-101) and the enum value
(include/qcu_enum.h:12), so parity is against the oracle's restatement:
CPU identities of the oracle, and GPU parity of the clover apply and of the
even-odd clover solves."""
import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import TOL, dev, rel

G5 = np.array([1, 1, -1, -1])  # gamma5 in the DeGrand-Rossi basis (chirality blocks)


def test_identity_clover_is_wilson():
    L, n = (4, 4, 2, 4), 3
    g = S.random_gauge(L, n, seed=1)
    x = S.random_fermions(L, n, 1, seed=2, parities=2)[0]
    one = np.broadcast_to(np.eye(2 * n), (2, S.half_volume(L), 2, 2 * n, 2 * n)).astype(np.complex128)
    assert rel(O.wilson_full(x, g, L, 0.12, clover=one), O.wilson_full(x, g, L, 0.12)) < 1e-14


def test_clover_hermitian_and_gamma5_hermiticity():
    L, n = (4, 4, 2, 4), 3
    g = S.random_gauge(L, n, seed=3)
    c = S.random_clover(L, n, eps=0.2, seed=4)
    psi = S.random_fermions(L, n, 2, seed=5)
    # A = A^dag
    assert rel(O.clover_apply(psi, c, L, 1, dagger=1), O.clover_apply(psi, c, L, 1, dagger=0)) < 1e-14
    # M^dag = gamma5 M gamma5 (A commutes with gamma5)
    x = S.random_fermions(L, n, 1, seed=6, parities=2)[0]
    g5 = G5[None, None, :, None]
    lhs = O.wilson_full(x, g, L, 0.11, dagger=1, clover=c)
    rhs = g5 * O.wilson_full(g5 * x, g, L, 0.11, clover=c)
    assert rel(lhs, rhs) < 1e-13


def test_clover_cgnr_converges():
    L, n = (4, 4, 2, 4), 3
    g = S.random_gauge(L, n, seed=7)
    c = S.random_clover(L, n, eps=0.2, seed=8)
    b = S.random_fermions(L, n, 1, seed=9, parities=2)[0]
    x, it, res = O.cgnr_full(b, g, L, 0.11, tol=1e-11, clover=c)
    assert res < 1e-11
    assert O.true_residual(x, b, g, L, 0.11, clover=c) < 1e-11


# ---- GPU ---------------------------------------------------------------------

def _resident(torch, Q, prec, nrhs, fields):
    db, nb = Q.field_bytes(prec, nrhs)
    buf = torch.empty(db // 8 + 2, dtype=torch.float64, device="cuda")
    nrm = torch.empty(nb // 4 + 4, dtype=torch.float32, device="cuda") if nb else None
    src = [dev(torch, f) for f in fields]
    Q.pack_fermions(buf.data_ptr(), nrm.data_ptr() if nrm is not None else None, [s.data_ptr() for s in src],
                    Q.QCU_SRC_EO_HALF, 0, prec)
    return buf, nrm, src


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [2, 1, 0, 4])
@pytest.mark.parametrize("n", [3, 4])
def test_clover_apply_and_inverse(cuda, qcu_lib, prec, n):
    torch, Q = cuda, qcu_lib
    L, nrhs = (4, 4, 4, 8), 4
    g = S.random_gauge(L, n, seed=20)
    c = S.random_clover(L, n, eps=0.1, seed=21)  # well conditioned: the inverses agree to rounding
    psi = S.random_fermions(L, n, nrhs, seed=22)
    Q.initGridSize(L, n)
    dg, dc = dev(torch, g), dev(torch, c)
    Q.loadQcuGauge(dg.data_ptr())
    Q.load_clover(dc.data_ptr())
    vh = S.half_volume(L)
    cinv = np.linalg.inv(c)  # per-site block inverses
    for parity in (0, 1):
        buf_in, n_in, keep = _resident(torch, Q, prec, nrhs, psi)
        db, nb = Q.field_bytes(prec, nrhs)
        out = torch.empty(db // 8 + 2, dtype=torch.float64, device="cuda")
        n_out = torch.empty(nb // 4 + 4, dtype=torch.float32, device="cuda") if nb else None
        for inverse, cl in ((0, c), (1, cinv)):
            Q.clover_mrhs(out.data_ptr(), n_out.data_ptr() if nb else None, buf_in.data_ptr(),
                          n_in.data_ptr() if nb else None, nrhs, parity, inverse, prec)
            outs = [torch.zeros((vh, 4, n), dtype=torch.complex128, device="cuda") for _ in range(nrhs)]
            Q.unpack_fermions([o.data_ptr() for o in outs], out.data_ptr(), n_out.data_ptr() if nb else None,
                              Q.QCU_SRC_EO_HALF, 0, prec)
            Q.synchronize()
            got = np.stack([o.cpu().numpy() for o in outs])
            assert rel(got, O.clover_apply(psi, cl, L, parity)) < TOL[prec], (parity, inverse)


@pytest.mark.gpu
@pytest.mark.parametrize("solver,inner", [(0, 2), (0, 1), (0, 0), (1, 1)])
def test_clover_solve(cuda, qcu_lib, solver, inner):
    """Even-odd Wilson-clover solve (Mhat = A_ee - kappa^2 D_eo A_oo^-1 D_oe)
    checked by the oracle's FP64 true residual of the full clover system."""
    torch, Q = cuda, qcu_lib
    L, n, kappa, tol, nrhs = (4, 4, 4, 8), 3, 0.115, 1e-10, 3
    g = S.random_gauge(L, n, seed=30)
    c = S.random_clover(L, n, eps=0.1, seed=31)  # min |eigenvalue of A| 0.45; eps = 0.2 gives 0.005
    b = S.random_fermions(L, n, nrhs, seed=32, parities=2)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(True)
    dg, dc = dev(torch, g), dev(torch, c)
    Q.loadQcuGauge(dg.data_ptr())
    Q.load_clover(dc.data_ptr())
    db = [dev(torch, b[r]) for r in range(nrhs)]
    dx = [torch.zeros_like(v) for v in db]
    p = Q.solver_params(kappa=kappa, tol=tol, inner_precision=inner, solver=solver, use_clover=1)
    Q.invert([x.data_ptr() for x in dx], [v.data_ptr() for v in db], p)
    for r in range(nrhs):
        x = dx[r].cpu().numpy()
        assert O.true_residual(x, b[r], g, L, kappa, antiperiodic_t=True, clover=c) < 2 * tol
        assert p.converged[r] == 1


@pytest.mark.gpu
def test_singular_clover_rejected(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L, n = (4, 4, 4, 4), 3
    Q.initGridSize(L, n)
    g = dev(torch, S.random_gauge(L, n, seed=40))
    Q.loadQcuGauge(g.data_ptr())
    c = S.random_clover(L, n, eps=0.1, seed=41)
    c[1, 5, 0] = 0.0  # one singular block
    dc = dev(torch, c)
    with pytest.raises(Q.QcuError) as e:
        Q.load_clover(dc.data_ptr())
    assert e.value.code == 2
