"""GPU tests of the even-odd preconditioned solves (cg_inverter and the MRHS
qcuInvert), checked by the FP64 oracle's true residual |b - M x| / |b| on the
full lattice (M = 1 - kappa D), computed independently on the CPU."""
import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import dev, rel

pytestmark = pytest.mark.gpu


def setup(torch, Q, L, n, seed, antiperiodic=True):
    g = S.random_gauge(L, n, seed=seed)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(antiperiodic)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    return g, dg


def solve(torch, Q, b, **kw):
    nrhs = b.shape[0]
    db = [dev(torch, b[r]) for r in range(nrhs)]
    dx = [torch.zeros_like(x) for x in db]
    p = Q.solver_params(**kw)
    Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    return np.stack([x.cpu().numpy() for x in dx]), p


@pytest.mark.parametrize("inner", [2, 1, 0, 4])
def test_cg_mrhs_all_precisions(cuda, qcu_lib, inner):
    torch, Q = cuda, qcu_lib
    L, n, kappa, tol = (4, 4, 4, 8), 3, 0.12, 1e-10
    g, _ = setup(torch, Q, L, n, 200)
    b = S.random_fermions(L, n, 4, seed=201, parities=2)
    x, p = solve(torch, Q, b, kappa=kappa, tol=tol, inner_precision=inner, solver=Q.QCU_SOLVER_CG)
    for r in range(4):
        assert p.converged[r] == 1
        res = O.true_residual(x[r], b[r], g, L, kappa, antiperiodic_t=True)
        assert res < 2 * tol, (r, res)
        assert abs(res - p.true_residual[r]) < 0.5 * tol + 0.1 * res
    if inner != 2:
        assert p.reliable_updates >= 1


@pytest.mark.parametrize("inner", [2, 1])
def test_bicgstab(cuda, qcu_lib, inner):
    torch, Q = cuda, qcu_lib
    L, n, kappa, tol = (4, 4, 4, 4), 3, 0.11, 1e-9
    g, _ = setup(torch, Q, L, n, 210)
    b = S.random_fermions(L, n, 3, seed=211, parities=2)
    x, p = solve(torch, Q, b, kappa=kappa, tol=tol, inner_precision=inner, solver=Q.QCU_SOLVER_BICGSTAB)
    for r in range(3):
        assert O.true_residual(x[r], b[r], g, L, kappa, antiperiodic_t=True) < 2 * tol


def test_point_sources_su4_lexicographic(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L, n, kappa, tol = (4, 4, 2, 4), 4, 0.11, 1e-10
    g, _ = setup(torch, Q, L, n, 220, antiperiodic=False)
    b = S.point_sources(L, n, 3, seed=221)
    blex = np.stack([O.eo_to_lex(b[r], L) for r in range(3)])
    xlex, p = solve(torch, Q, blex, kappa=kappa, tol=tol, inner_precision=1, src_mode=Q.QCU_SRC_LEX)
    for r in range(3):
        x = O.lex_to_eo(xlex[r], L)
        assert O.true_residual(x, b[r], g, L, kappa) < 2 * tol


def test_masks_uneven_rhs(cuda, qcu_lib):
    """RHS of very different difficulty (a zero source, a scaled copy) all
    converge; converged RHS are masked while the rest iterate."""
    torch, Q = cuda, qcu_lib
    L, n, kappa, tol = (4, 4, 4, 4), 3, 0.124, 1e-10
    g, _ = setup(torch, Q, L, n, 230)
    b = S.random_fermions(L, n, 4, seed=231, parities=2)
    b[1] = 0.0
    b[1, 0, 0, 0, 0] = 1e-3  # tiny point source
    b[2] = 1e6 * b[3]
    x, p = solve(torch, Q, b, kappa=kappa, tol=tol, inner_precision=1)
    for r in range(4):
        assert O.true_residual(x[r], b[r], g, L, kappa, antiperiodic_t=True) < 2 * tol
    assert rel(x[2], 1e6 * x[3]) < 1e-8


@pytest.mark.parametrize("inner", [1, 0])
def test_slot_independence(cuda, qcu_lib, inner):
    """A slot's iterates do not depend on what the other slots hold: RHS 0 of
    [bX, bY, bY'] and of [bX, bZ, bZ'] are solved bit-identically, although
    the other slots take different iteration counts and reliable-update
    times (which restart those slots in the middle of RHS 0's solve)."""
    torch, Q = cuda, qcu_lib
    L, n, kappa, tol = (4, 4, 4, 8), 3, 0.12, 1e-10
    setup(torch, Q, L, n, 235)
    b = S.random_fermions(L, n, 5, seed=236, parities=2)
    b[2] *= 1e-4
    b[4, :, :4] = 0.0  # a source with a different spectrum
    x1, p1 = solve(torch, Q, b[[0, 1, 2]], kappa=kappa, tol=tol, inner_precision=inner)
    x2, p2 = solve(torch, Q, b[[0, 3, 4]], kappa=kappa, tol=tol, inner_precision=inner)
    assert p1.converged[0] == 1 and p2.converged[0] == 1
    assert np.array_equal(x1[0], x2[0])
    assert p1.true_residual[0] == p2.true_residual[0]


def test_graph_and_eager_agree(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L, n, kappa = (4, 4, 4, 4), 3, 0.12
    setup(torch, Q, L, n, 240)
    b = S.random_fermions(L, n, 2, seed=241, parities=2)
    x1, p1 = solve(torch, Q, b, kappa=kappa, tol=1e-10, use_graph=1)
    x2, p2 = solve(torch, Q, b, kappa=kappa, tol=1e-10, use_graph=0)
    assert p1.iterations == p2.iterations
    assert np.array_equal(x1, x2)


def test_cg_inverter_abi(cuda, qcu_lib):
    """The reference's cg_inverter entry point (an empty stub there)."""
    torch, Q = cuda, qcu_lib
    L, kappa, tol = (4, 4, 4, 8), 0.12, 1e-10
    g = S.random_gauge(L, 3, seed=250)
    b = S.random_fermions(L, 3, 1, seed=251, parities=2)[0]
    Q.set_antiperiodic_t(False)
    dg, dbv = dev(torch, g), dev(torch, b)
    dx = torch.zeros_like(dbv)
    Q.cg_inverter(dx.data_ptr(), dbv.data_ptr(), dg.data_ptr(), L, tol, kappa)
    x = dx.cpu().numpy()
    assert O.true_residual(x, b, g, L, kappa) < 2 * tol
    # agrees with the oracle's own CGNR solution
    xo, _, _ = O.cgnr_full(b, g, L, kappa, tol=1e-12)
    assert rel(x, xo) < 1e-8


def test_gamma5_hermiticity_of_schur_operator(cuda, qcu_lib):
    """<y, Mhat x> = <Mhat^dag y, x> with Mhat^dag built from the f=-1 hop."""
    torch, Q = cuda, qcu_lib
    L, n, kappa = (4, 4, 4, 4), 3, 0.12
    g, _ = setup(torch, Q, L, n, 260)
    x = S.random_fermions(L, n, 1, seed=261)
    y = S.random_fermions(L, n, 1, seed=262)

    def mhat(v, dag):
        vh = S.half_volume(L)
        db, nb = Q.field_bytes(2, 1)
        bufs = [torch.zeros(db // 8, dtype=torch.float64, device="cuda") for _ in range(3)]
        src = dev(torch, v[0])
        Q.pack_fermions(bufs[0].data_ptr(), None, [src.data_ptr()], Q.QCU_SRC_EO_HALF, 0, 2)
        Q.dslash_mrhs(bufs[1].data_ptr(), None, bufs[0].data_ptr(), None, 1, 1, dag, 2)
        Q.dslash_xpay_mrhs(bufs[2].data_ptr(), None, bufs[1].data_ptr(), None, bufs[0].data_ptr(), None, 1, 0, dag,
                           2, -kappa * kappa, 1.0)
        out = torch.zeros((vh, 4, n), dtype=torch.complex128, device="cuda")
        Q.unpack_fermions([out.data_ptr()], bufs[2].data_ptr(), None, Q.QCU_SRC_EO_HALF, 0, 2)
        Q.synchronize()
        return out.cpu().numpy()[None]

    lhs = np.vdot(y, mhat(x, 0))
    rhs = np.vdot(mhat(y, 1), x)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


@pytest.mark.parametrize("variant", [1, 4])
def test_bicgstab_bf16_tensor_core_masks(cuda, qcu_lib, variant):
    """BiCGStab with BF16 inner dslash on the tensor cores (SU(4), 16 RHS, one
    source 1e-4 times smaller, one zero) to 1e-8, checked by the oracle's
    FP64 true residual: the masked tensor-core epilogue inside the solver."""
    import os
    torch, Q = cuda, qcu_lib
    L, n, kappa, tol, nrhs = (4, 4, 4, 8), 4, 0.11, 1e-8, 16
    g, _ = setup(torch, Q, L, n, 250)
    b = S.random_fermions(L, n, nrhs, seed=251, parities=2)
    b[1] *= 1e-4
    b[2] = 0.0
    os.environ["QCU_DSLASH_CONFIG"] = "1,0,0,0,0,0,%d" % variant
    try:
        x, p = solve(torch, Q, b, kappa=kappa, tol=tol, inner_precision=4, solver=Q.QCU_SOLVER_BICGSTAB)
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]
    for r in range(nrhs):
        assert p.converged[r] == 1
        if r != 2:
            assert O.true_residual(x[r], b[r], g, L, kappa, antiperiodic_t=True) < 2 * tol
    assert not np.any(x[2])
