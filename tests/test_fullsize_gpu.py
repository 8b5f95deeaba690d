"""GPU parity at the benchmarked sizes, against the FP64 oracle.

* 32^3 x 64 SU(3) dslash (the headline lattice) in FP64, FP16 and BF16 at
  nrhs = 12 and in FP32 at nrhs = 1, 4 and 24: two basis RHS go through the
  oracle and every RHS is a combination of them, so all RHS are checked by
  linearity while the oracle runs on two.
* The mixed-precision eo-CG of the solve benchmark (24^3 x 48 SU(3),
  nrhs = 12, kappa = 0.12, point sources, tolerance 1e-10), FP32 and FP16
  inner, each RHS checked by the oracle's FP64 true residual of the full
  Wilson system.
* 16x16x12x32 SU(3), nrhs 128 (fields larger than L2): the register
  kernel's slab site order, bit-identical across slab heights.
* 16^3 x 32 SU(N), N = 4, 6, 8, nrhs 16 / 32 / 64: the CUDA-core kernels
  (FP32, BF16) and the tensor-core kernels (BF16, component- and site-major
  fields), and a masked BiCGStab to 1e-8 (one source 1e-4 smaller, one
  zero) checked RHS by RHS.

Tolerances (relative L2): 1e-13 FP64, 1e-6 FP32, 5e-3 FP16/BF16; solves:
the oracle's true residual at most 2x the requested tolerance."""
import os

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import TOL, dev

pytestmark = pytest.mark.gpu

L_BIG = (32, 32, 32, 64)
L_SUN = (16, 16, 16, 32)


@pytest.fixture(scope="module")
def big_gauge():
    return S.random_gauge(L_BIG, 3, seed=140)


_sun_gauges = {}


def sun_gauge(n):
    if n not in _sun_gauges:
        _sun_gauges.clear()  # one N at a time keeps host memory small
        _sun_gauges[n] = S.random_gauge(L_SUN, n, seed=300 + n)
    return _sun_gauges[n]


def linear_check(torch, Q, g, L, n, prec, nrhs, seed, parity=1, dagger=0):
    """Apply D through the drop-in ABI to nrhs RHS that are combinations of
    two seeded Gaussian bases; return each RHS's relative L2 error against
    the same combination of the oracle's results on the bases.  The inputs
    and the comparison stay on the device."""
    vh = S.half_volume(L)
    rng = np.random.default_rng(seed)
    base = (rng.standard_normal((2, vh, 4, n)) + 1j * rng.standard_normal((2, vh, 4, n))) * np.sqrt(0.5)
    coef = rng.standard_normal((nrhs, 2))
    ref = O.dslash(base, g, L, parity, dagger, True)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(True)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    del dg
    Q.getDslash(Q.DSLASH_WILSON, 0.0, n, nrhs, prec)
    db, dref = dev(torch, base), dev(torch, ref)
    ins = [float(coef[r, 0]) * db[0] + float(coef[r, 1]) * db[1] for r in range(nrhs)]
    outs = [torch.zeros_like(x) for x in ins]
    for r in range(nrhs):
        Q.pushBackFermions(outs[r].data_ptr(), ins[r].data_ptr())
    Q.startDslash(parity, dagger)
    torch.cuda.synchronize()
    errs = []
    for r in range(nrhs):
        want = float(coef[r, 0]) * dref[0] + float(coef[r, 1]) * dref[1]
        errs.append(float(torch.linalg.vector_norm(outs[r] - want) / torch.linalg.vector_norm(want)))
    del ins, outs, db, dref
    torch.cuda.empty_cache()
    return errs


@pytest.mark.parametrize("prec,nrhs", [(2, 12), (0, 12), (4, 12), (1, 1), (1, 4), (1, 24)])
def test_headline_lattice_every_precision(cuda, qcu_lib, big_gauge, prec, nrhs):
    """32^3 x 64 SU(3): the autotuned kernel of each precision and RHS count
    (the 32-bit element offsets of the register kernels are exercised up to
    12 * 24 * 2^20 elements per field at nrhs = 24)."""
    errs = linear_check(cuda, qcu_lib, big_gauge, L_BIG, 3, prec, nrhs, seed=141 + nrhs + 10 * prec)
    assert max(errs) < TOL[prec], (prec, nrhs, max(errs))


@pytest.mark.parametrize("inner", [1, 0])
def test_solve_benchmark_workload(cuda, qcu_lib, inner):
    """24^3 x 48 SU(3), nrhs = 12, kappa = 0.12, point sources, tolerance
    1e-10: FP32 / FP16 inner iterations with FP64 reliable updates; every RHS
    meets the tolerance by the oracle's FP64 true residual."""
    torch, Q = cuda, qcu_lib
    L, n, nrhs, kappa, tol = (24, 24, 24, 48), 3, 12, 0.12, 1e-10
    g = S.random_gauge(L, n, seed=5)
    b = S.point_sources(L, n, nrhs, seed=6)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(True)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    db = [dev(torch, b[r]) for r in range(nrhs)]
    dx = [torch.zeros_like(x) for x in db]
    p = Q.solver_params(kappa=kappa, tol=tol, inner_precision=inner, max_iter=20000)
    Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    for r in range(nrhs):
        assert p.converged[r]
        res = O.true_residual(dx[r].cpu().numpy(), b[r], g, L, kappa, antiperiodic_t=True)
        assert res < 2 * tol, (inner, r, res)


# (kernel name, storage precision, QCU_DSLASH_CONFIG pin or None for the autotuner)
SUN_KERNELS = [("cuda_core_fp32", 1, None), ("cuda_core_bf16", 4, "2,64,1,0"),
               ("tensor_core_projected", 4, "1,0,0,0,0,0,1"), ("tensor_core_projected_tma", 4, "1,0,0,0,0,0,2"),
               ("tensor_core_spinor", 4, "1,0,0,0,0,0,4"), ("tensor_core_spinor_ring5", 4, "1,0,0,0,0,0,6"),
               ("tensor_core_spinor_site_major", 5, "1,0,0,0,0,0,4"),
               ("tensor_core_spinor_site_major_ring5", 5, "1,0,0,0,0,0,6"),
               ("tensor_core_site_major_tuned", 5, None)]


@pytest.mark.parametrize("nrhs", [16, 32, 64])
@pytest.mark.parametrize("n", [4, 6, 8])
@pytest.mark.parametrize("kernel", SUN_KERNELS, ids=[k[0] for k in SUN_KERNELS])
def test_sun_benchmark_lattice(cuda, qcu_lib, kernel, n, nrhs):
    """16^3 x 32 SU(N): each benchmarked kernel against the oracle at the
    benchmarked N and RHS counts (both parities checked through D_eo and
    D_oe^dag)."""
    name, prec, pin = kernel
    if pin:
        os.environ["QCU_DSLASH_CONFIG"] = pin
    try:
        for parity, dagger in ((0, 0), (1, 1)):
            errs = linear_check(cuda, qcu_lib, sun_gauge(n), L_SUN, n, prec, nrhs, seed=400 + nrhs + n,
                                parity=parity, dagger=dagger)
            assert max(errs) < TOL[prec], (name, n, nrhs, parity, max(errs))
    finally:
        os.environ.pop("QCU_DSLASH_CONFIG", None)


@pytest.mark.parametrize("inner", [1, 4])
@pytest.mark.parametrize("n", [4, 6, 8])
def test_sun_bicgstab_masks(cuda, qcu_lib, n, inner):
    """Masked BiCGStab of the SU(N) benchmark: 16 RHS on 16^3 x 32, kappa
    0.11, tolerance 1e-8, one source 1e-4 times smaller and one zero; FP32
    and BF16 inner.  Every RHS converges to the tolerance by the oracle's
    true residual, and the zero source gives the zero solution."""
    torch, Q = cuda, qcu_lib
    nr, kappa, tol = 16, 0.11, 1e-8
    g = sun_gauge(n)
    b = S.random_fermions(L_SUN, n, nr, seed=302, parities=2)
    b[1] *= 1e-4
    b[2] = 0
    Q.initGridSize(L_SUN, n)
    Q.set_antiperiodic_t(True)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    db = [dev(torch, b[r]) for r in range(nr)]
    dx = [torch.zeros_like(x) for x in db]
    p = Q.solver_params(kappa=kappa, tol=tol, inner_precision=inner, solver=Q.QCU_SOLVER_BICGSTAB, max_iter=5000)
    Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    assert float(dx[2].abs().max()) == 0.0
    for r in range(nr):
        assert p.converged[r], r
        if r == 2:
            continue
        res = O.true_residual(dx[r].cpu().numpy(), b[r], g, L_SUN, kappa, antiperiodic_t=True)
        assert res < 2 * tol, (n, inner, r, res)


@pytest.mark.parametrize("prec", [1, 4])
def test_slab_site_order_bit_identical(cuda, qcu_lib, prec):
    """16x16x12x32 SU(3), nrhs 128 (fields of 604 MB FP32, larger than L2):
    the register kernel walks the lattice in slabs of z-planes (6 by the
    host's rule here).  The result is bit-identical in the field's own order
    and in slabs of 3 and 2 planes, and meets the oracle's tolerance (two
    basis RHS checked, the rest by linearity)."""
    torch, Q = cuda, qcu_lib
    L, n, nrhs = (16, 16, 12, 32), 3, 128
    g = S.random_gauge(L, n, seed=700)
    got = {}
    try:
        for zs in (None, "0", "3", "2"):
            if zs is None:
                os.environ.pop("QCU_DSLASH_ZSLAB", None)
            else:
                os.environ["QCU_DSLASH_ZSLAB"] = zs
            errs, outs = linear_check_outputs(torch, Q, g, L, n, prec, nrhs, seed=701)
            assert max(errs) < TOL[prec], (zs, max(errs))
            got[zs] = outs
    finally:
        os.environ.pop("QCU_DSLASH_ZSLAB", None)
    for zs in ("0", "3", "2"):
        assert all(torch.equal(a, b) for a, b in zip(got[None], got[zs])), zs


def linear_check_outputs(torch, Q, g, L, n, prec, nrhs, seed):
    """As linear_check, also returning the output fields (on the device)."""
    vh = S.half_volume(L)
    rng = np.random.default_rng(seed)
    base = (rng.standard_normal((2, vh, 4, n)) + 1j * rng.standard_normal((2, vh, 4, n))) * np.sqrt(0.5)
    coef = rng.standard_normal((nrhs, 2))
    ref = O.dslash(base, g, L, 1, 0, True)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(True)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    del dg
    Q.getDslash(Q.DSLASH_WILSON, 0.0, n, nrhs, prec)
    db, dref = dev(torch, base), dev(torch, ref)
    ins = [float(coef[r, 0]) * db[0] + float(coef[r, 1]) * db[1] for r in range(nrhs)]
    outs = [torch.zeros_like(x) for x in ins]
    for r in range(nrhs):
        Q.pushBackFermions(outs[r].data_ptr(), ins[r].data_ptr())
    Q.startDslash(1, 0)
    torch.cuda.synchronize()
    errs = []
    for r in range(nrhs):
        want = float(coef[r, 0]) * dref[0] + float(coef[r, 1]) * dref[1]
        errs.append(float(torch.linalg.vector_norm(outs[r] - want) / torch.linalg.vector_norm(want)))
    del ins, db, dref
    return errs, outs
