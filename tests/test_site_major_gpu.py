"""GPU tests of the site-major BF16 storage (QCU_BF16_SITE_PRECISION): fields
[Vh][4N][nrhs] whose dslash is the spinor-operand tensor-core kernel.

* pack writes exactly the component-major BF16 values, transposed to the
  site-major order (bitwise), and unpack inverts it;
* the dslash on site-major fields is bit-identical to the same tensor-core
  variant on component-major fields (the same MMA operands in the same
  order) and meets the BF16 tolerance against the FP64 oracle;
* the xpay epilogue, the drop-in ABI (getDslash with this precision), and a
  mixed-precision solve with site-major inner fields (masked BiCGStab and
  CG, checked RHS by RHS with the oracle's FP64 true residual);
* the cases the layout does not take are refused with QCU_ERR_UNSUPPORTED
  (RHS counts that are not a multiple of 4)."""
import os

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import TOL, abi_dslash, dev, rel

pytestmark = pytest.mark.gpu
SITE = 5  # QCU_BF16_SITE_PRECISION
BF16 = 4


def _fields(torch, Q, nrhs, prec, count):
    db, _ = Q.field_bytes(prec, nrhs)
    return [torch.zeros(db // 2 + 8, dtype=torch.int16, device="cuda") for _ in range(count)]


def _setup(torch, Q, L, n, g):
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(True)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    return dg


@pytest.mark.parametrize("n,nrhs", [(3, 4), (4, 12), (8, 36)])
def test_pack_is_the_transposed_component_major_field(cuda, qcu_lib, n, nrhs):
    torch, Q = cuda, qcu_lib
    L = (4, 4, 2, 6)
    vh = S.half_volume(L)
    dg = _setup(torch, Q, L, n, S.random_gauge(L, n, seed=500))
    psi = S.random_fermions(L, n, nrhs, seed=501)
    src = [dev(torch, psi[r]) for r in range(nrhs)]
    ptrs = [s.data_ptr() for s in src]
    comp, site = _fields(torch, Q, nrhs, BF16, 1)[0], _fields(torch, Q, nrhs, SITE, 1)[0]
    Q.pack_fermions(comp.data_ptr(), None, ptrs, Q.QCU_SRC_EO_HALF, 1, BF16)
    Q.pack_fermions(site.data_ptr(), None, ptrs, Q.QCU_SRC_EO_HALF, 1, SITE)
    Q.synchronize()
    words = 4 * n * vh * nrhs * 2  # two BF16 per complex
    c = comp[:words].cpu().numpy().reshape(4 * n, vh, nrhs, 2)
    s = site[:words].cpu().numpy().reshape(vh, 4 * n, nrhs, 2)
    assert np.array_equal(c.transpose(1, 0, 2, 3), s)
    outs = [torch.zeros_like(x) for x in src]
    Q.unpack_fermions([o.data_ptr() for o in outs], site.data_ptr(), None, Q.QCU_SRC_EO_HALF, 1, SITE)
    back = [torch.zeros_like(x) for x in src]
    Q.unpack_fermions([o.data_ptr() for o in back], comp.data_ptr(), None, Q.QCU_SRC_EO_HALF, 1, BF16)
    Q.synchronize()
    for r in range(nrhs):
        assert torch.equal(outs[r], back[r])
    assert rel(np.stack([o.cpu().numpy() for o in outs]), psi) < 5e-3
    del dg


@pytest.mark.parametrize("variant", [4, 5, 6, 7, 8])
@pytest.mark.parametrize("n,nrhs", [(3, 4), (4, 16), (6, 32), (8, 64), (5, 36), (8, 8), (7, 12)])
def test_dslash_site_major_bitwise_and_oracle(cuda, qcu_lib, n, nrhs, variant):
    """Both parities and dagger flags, antiperiodic t; RHS counts that fill
    the 128 MMA rows, leave them partly empty or end inside the second 32-RHS
    box; the site-major result equals the component-major one bit for bit."""
    torch, Q = cuda, qcu_lib
    L = (4, 4, 4, 8)
    g = S.random_gauge(L, n, seed=510 + n)
    psi = S.random_fermions(L, n, nrhs, seed=511)
    # variants 7-8 take tiles of at most 32 RHS; larger tiles run the first variant that fits (4)
    ran = variant if variant <= 6 or nrhs <= 32 else 4
    try:
        for parity, dag in ((0, 0), (1, 1), (1, 0)):
            os.environ["QCU_DSLASH_CONFIG"] = "1,0,0,0,0,0,%d" % variant
            got = abi_dslash(torch, Q, psi, g, L, parity, dag, SITE, antiperiodic_t=True)
            assert Q.last_dslash_shape()[3] == -ran
            assert rel(got, O.dslash(psi, g, L, parity, dag, True)) < TOL[BF16], (parity, dag)
            os.environ["QCU_DSLASH_CONFIG"] = "1,0,0,0,0,0,%d" % ran
            other = abi_dslash(torch, Q, psi, g, L, parity, dag, BF16, antiperiodic_t=True)
            assert Q.last_dslash_shape()[3] == -ran
            assert np.array_equal(got, other), (parity, dag)
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]


def test_tuned_site_major_is_a_tensor_core_shape(cuda, qcu_lib):
    """The autotuner's choice for site-major fields is one of the
    spinor-operand variants, and the kernel list names only those."""
    torch, Q = cuda, qcu_lib
    L, n, nrhs = (4, 4, 4, 8), 4, 16
    dg = _setup(torch, Q, L, n, S.random_gauge(L, n, seed=520))
    assert Q.tune_dslash(nrhs, SITE)[4] in (-4, -5, -6, -7, -8)
    assert sorted(k[3] for k in Q.dslash_kernels(SITE, n)) == [-8, -7, -6, -5, -4]
    del dg


def test_xpay_resident_site_major(cuda, qcu_lib):
    """qcuPackFermions -> qcuDslashXpayMRHS -> qcuUnpackFermions on site-major
    fields, with per-call a and b: bit-identical to component-major BF16."""
    torch, Q = cuda, qcu_lib
    L, n, nrhs = (4, 4, 4, 8), 4, 12
    g = S.random_gauge(L, n, seed=530)
    full = S.random_fermions(L, n, nrhs, seed=531, parities=2)
    dg = _setup(torch, Q, L, n, g)
    src_o = [dev(torch, full[r, 1]) for r in range(nrhs)]
    src_e = [dev(torch, full[r, 0]) for r in range(nrhs)]
    a, b = -0.0144, 1.0
    res = {}
    for prec in (SITE, BF16):
        f = _fields(torch, Q, nrhs, prec, 3)
        Q.pack_fermions(f[0].data_ptr(), None, [s.data_ptr() for s in src_o], Q.QCU_SRC_EO_HALF, 1, prec)
        Q.pack_fermions(f[1].data_ptr(), None, [s.data_ptr() for s in src_e], Q.QCU_SRC_EO_HALF, 0, prec)
        Q.dslash_xpay_mrhs(f[2].data_ptr(), None, f[0].data_ptr(), None, f[1].data_ptr(), None, nrhs, 0, 0, prec, a, b)
        outs = [torch.zeros_like(s) for s in src_e]
        Q.unpack_fermions([o.data_ptr() for o in outs], f[2].data_ptr(), None, Q.QCU_SRC_EO_HALF, 0, prec)
        Q.synchronize()
        res[prec] = np.stack([o.cpu().numpy() for o in outs])
    want = a * O.dslash(full[:, 1], g, L, 0, 0, True) + b * full[:, 0]
    assert rel(res[SITE], want) < TOL[BF16]
    assert np.array_equal(res[SITE], res[BF16])
    del dg


@pytest.mark.parametrize("solver", [0, 1])
def test_solve_with_site_major_inner_fields(cuda, qcu_lib, solver):
    """Masked mixed-precision eo solves (CG, BiCGStab) with site-major BF16
    inner fields: 8 RHS on 4^3 x 8 SU(4), kappa 0.11, tolerance 1e-8, one
    source 1e-4 smaller and one zero; every RHS meets the tolerance by the
    oracle's FP64 true residual and the zero source gives zero."""
    torch, Q = cuda, qcu_lib
    L, n, nr, kappa, tol = (4, 4, 4, 8), 4, 8, 0.11, 1e-8
    g = S.random_gauge(L, n, seed=540)
    b = S.random_fermions(L, n, nr, seed=541, parities=2)
    b[1] *= 1e-4
    b[2] = 0
    dg = _setup(torch, Q, L, n, g)
    db = [dev(torch, b[r]) for r in range(nr)]
    dx = [torch.zeros_like(x) for x in db]
    p = Q.solver_params(kappa=kappa, tol=tol, inner_precision=SITE, solver=solver, max_iter=5000)
    Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    assert float(dx[2].abs().max()) == 0.0
    for r in range(nr):
        assert p.converged[r], r
        if r != 2:
            res = O.true_residual(dx[r].cpu().numpy(), b[r], g, L, kappa, antiperiodic_t=True)
            assert res < 2 * tol, (solver, r, res)
    del dg


def test_site_major_refusals(cuda, qcu_lib):
    """RHS counts that are not a multiple of 4 (a dslash, a solve) are
    refused with QCU_ERR_UNSUPPORTED, and the library stays usable."""
    torch, Q = cuda, qcu_lib
    L, n = (4, 4, 4, 8), 3
    g = S.random_gauge(L, n, seed=550)
    psi = S.random_fermions(L, n, 6, seed=551)
    with pytest.raises(Q.QcuError) as e:
        abi_dslash(torch, Q, psi, g, L, 1, 0, SITE, antiperiodic_t=True)
    assert e.value.code == 3  # QCU_ERR_UNSUPPORTED
    Q.clear_error()
    b = S.random_fermions(L, n, 6, seed=552, parities=2)
    dg = _setup(torch, Q, L, n, g)
    db = [dev(torch, b[r]) for r in range(6)]
    dx = [torch.zeros_like(x) for x in db]
    with pytest.raises(Q.QcuError) as e:
        Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db],
                 Q.solver_params(kappa=0.11, tol=1e-8, inner_precision=SITE))
    assert e.value.code == 3  # QCU_ERR_UNSUPPORTED
    Q.clear_error()
    got = abi_dslash(torch, Q, psi[:4], g, L, 1, 0, SITE, antiperiodic_t=True)
    assert rel(got, O.dslash(psi[:4], g, L, 1, 0, True)) < TOL[BF16]
    del dg
