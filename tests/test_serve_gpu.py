"""GPU tests of the solve server: continuous MRHS batching over resident
gauges.  Every result is checked by the oracle's FP64 true residual, and a
request's solution is the same solved alone and solved in a mix of
concurrent requests on two gauges, within what the requested tolerance
allows.  A slot's iteration never reads another slot's data, but the
reduction order of its inner products depends on its slot position."""
import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import dev, rel

pytestmark = pytest.mark.gpu


def fields(torch, b):
    db = [dev(torch, b[r]) for r in range(b.shape[0])]
    dx = [torch.zeros_like(x) for x in db]
    return db, dx


def test_alone_and_in_mix(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    LA, nA = (4, 4, 4, 8), 3
    LB, nB = (4, 4, 4, 4), 4
    gA, gB = S.random_gauge(LA, nA, seed=500), S.random_gauge(LB, nB, seed=501)
    dgA, dgB = dev(torch, gA), dev(torch, gB)
    srv = Q.Server(8 << 30, max_slots=12, inner_precision=Q.QCU_SINGLE_PRECISION)
    srv.add_gauge(0, LA, nA, dgA.data_ptr(), antiperiodic_t=True)
    srv.add_gauge(1, LB, nB, dgB.data_ptr(), antiperiodic_t=False)

    bX = S.random_fermions(LA, nA, 3, seed=502, parities=2)
    kX, tX = 0.118, 1e-10
    dbX, dxX = fields(torch, bX)
    info = srv.wait(srv.submit(0, kX, tX, [x.data_ptr() for x in dxX], [b.data_ptr() for b in dbX]))
    assert info.done and info.status == 0 and info.all_converged
    x_alone = np.stack([x.cpu().numpy() for x in dxX])

    # the mix: X again, arriving while other requests on both gauges run
    rng = np.random.default_rng(503)
    jobs = []
    for i in range(6):
        gid = i % 2
        L, n = (LA, nA) if gid == 0 else (LB, nB)
        nr = int(rng.integers(1, 5))
        b = S.random_fermions(L, n, nr, seed=510 + i, parities=2)
        kappa = float(rng.uniform(0.10, 0.125))
        tol = [1e-8, 1e-10, 1e-12][i % 3]
        db, dx = fields(torch, b)
        rid = srv.submit(gid, kappa, tol, [x.data_ptr() for x in dx], [v.data_ptr() for v in db])
        jobs.append((rid, gid, b, kappa, tol, dx, db))
        if i == 2:
            dbX2, dxX2 = fields(torch, bX)
            ridX = srv.submit(0, kX, tX, [x.data_ptr() for x in dxX2], [v.data_ptr() for v in dbX2])
    for rid, gid, b, kappa, tol, dx, db in jobs:
        info = srv.wait(rid)
        assert info.done and info.status == 0, (rid, info.status)
        L, g = (LA, gA) if gid == 0 else (LB, gB)
        for r in range(b.shape[0]):
            res = O.true_residual(dx[r].cpu().numpy(), b[r], g, L, kappa, antiperiodic_t=(gid == 0))
            assert res < 2 * tol, (rid, r, res, tol)
    info = srv.wait(ridX)
    assert info.done and info.status == 0
    x_mix = np.stack([x.cpu().numpy() for x in dxX2])
    # In the mix X occupies other slot positions, so the per-RHS reduction
    # trees (and with them the CG paths) differ at rounding level; each
    # solution has |b - M x| / |b| <= tol, so they differ by at most
    # 2 cond(M) tol (cond(M) is O(1) for these kappa on a random gauge).
    assert rel(x_mix, x_alone) < 20 * tX
    for r in range(3):
        assert O.true_residual(x_mix[r], bX[r], gA, LA, kX, antiperiodic_t=True) < 2 * tX
    st = srv.stats()
    assert st.completed == 8 and st.p99_s >= st.p50_s > 0
    srv.close()


def test_hbm_budget_admission(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L, n = (4, 4, 4, 8), 3
    g = dev(torch, S.random_gauge(L, n, seed=520))
    srv = Q.Server(1 << 16, max_slots=4)  # 64 KiB: not even the gauge fits
    with pytest.raises(Q.QcuError) as e:
        srv.add_gauge(0, L, n, g.data_ptr())
    assert e.value.code == 11
    srv.close()
    srv = Q.Server(64 << 20, max_slots=4)
    srv.add_gauge(0, L, n, g.data_ptr())
    assert 0 < srv.stats().hbm_used <= 64 << 20
    b = S.random_fermions(L, n, 5, seed=521, parities=2)
    db, dx = fields(torch, b)
    with pytest.raises(Q.QcuError) as e:  # more RHS than slots
        srv.submit(0, 0.12, 1e-10, [x.data_ptr() for x in dx], [v.data_ptr() for v in db])
    assert e.value.code == 11
    srv.close()


def test_site_major_bf16_inner_lanes(cuda, qcu_lib):
    """Server lanes with site-major BF16 inner fields (the tensor-core dslash,
    graph-captured solver chunks): requests of 1-7 RHS on an SU(4) and an
    SU(3) gauge (slot capacity 8, a multiple of 4) reach their tolerances by
    the oracle's FP64 true residual."""
    torch, Q = cuda, qcu_lib
    gauges = {0: ((4, 4, 4, 8), 4), 1: ((4, 4, 4, 4), 3)}
    g = {k: S.random_gauge(L, n, seed=560 + k) for k, (L, n) in gauges.items()}
    dg = {k: dev(torch, g[k]) for k in g}
    srv = Q.Server(8 << 30, max_slots=8, inner_precision=Q.QCU_BF16_SITE_PRECISION)
    for k, (L, n) in gauges.items():
        srv.add_gauge(k, L, n, dg[k].data_ptr(), antiperiodic_t=True)
    rng = np.random.default_rng(561)
    jobs = []
    for i in range(5):
        gid = i % 2
        L, n = gauges[gid]
        nr = int(rng.integers(1, 8))
        b = S.random_fermions(L, n, nr, seed=570 + i, parities=2)
        kappa, tol = float(rng.uniform(0.10, 0.12)), [1e-8, 1e-10][i % 2]
        db, dx = fields(torch, b)
        jobs.append((srv.submit(gid, kappa, tol, [x.data_ptr() for x in dx], [v.data_ptr() for v in db]),
                     gid, b, kappa, tol, dx, db))
    for rid, gid, b, kappa, tol, dx, db in jobs:
        info = srv.wait(rid)
        assert info.done and info.status == 0, (rid, info.status)
        L, _ = gauges[gid]
        for r in range(b.shape[0]):
            res = O.true_residual(dx[r].cpu().numpy(), b[r], g[gid], L, kappa, antiperiodic_t=True)
            assert res < 2 * tol, (rid, r, res)
    srv.close()
