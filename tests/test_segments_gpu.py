"""One launch over a work list of lattices (qcuDslashSegments) against one
launch per lattice: segments of different lattices, gauges and RHS counts,
with the same pinned kernel shape, give bit-identical results to the
library's own per-lattice dslash (qcuDslashMRHS on a session of that
lattice), and match the FP64 oracle.  A shape the segments do not fit
(an odd RHS count for R = 2) falls back to one launch per segment."""
import os

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import TOL, dev, rel

pytestmark = pytest.mark.gpu

LATTICES = [((8, 8, 8, 8), 12), ((4, 4, 4, 8), 4), ((8, 4, 6, 4), 6), ((4, 6, 4, 8), 2)]


def coalesced_gauge(torch, g, prec):
    """[4][2][Vh][3][3] complex128 caller gauge -> the coalesced [4][2][9][Vh] layout in `prec`, and the
    two-row copy in groups of 32 sites, [4][2][Vp/32][6][32] (Vp = Vh padded to 32)"""
    vh = g.shape[2]
    c = torch.from_numpy(np.ascontiguousarray(g.reshape(4, 2, vh, 9).transpose(0, 1, 3, 2))).cuda()
    c = c.to(torch.complex64 if prec == 1 else torch.complex128).contiguous()
    vp = (vh + 31) // 32 * 32
    t = torch.zeros((4, 2, 6, vp), dtype=c.dtype, device=c.device)
    t[..., :vh] = c[:, :, :6, :]
    return c, t.view(4, 2, 6, vp // 32, 32).permute(0, 1, 3, 2, 4).contiguous()


@pytest.mark.parametrize("prec,pin", [(1, "2,64,2,1,0,0,0,1"), (1, "2,128,2,0,0,0,0,0"), (2, "1,64,1,0,0,0,0,1")])
def test_work_list_matches_per_lattice_launches(cuda, qcu_lib, prec, pin):
    torch, Q = cuda, qcu_lib
    os.environ["QCU_DSLASH_CONFIG"] = pin
    try:
        segs, refs, keep, data = [], [], [], []
        for k, (L, nrhs) in enumerate(LATTICES):
            g = S.random_gauge(L, 3, seed=900 + k)
            psi = S.random_fermions(L, 3, nrhs, seed=910 + k)
            parity, dagger = k % 2, (k // 2) % 2
            # the library's per-lattice launch on its own session
            Q.initGridSize(L, 3)
            Q.set_antiperiodic_t(True)
            dg = dev(torch, g)
            Q.loadQcuGauge(dg.data_ptr())
            src = [dev(torch, psi[r]) for r in range(nrhs)]
            db, _ = Q.field_bytes(prec, nrhs)
            fin = torch.zeros(db // 8 + 2, dtype=torch.float64, device="cuda")
            fref = torch.zeros_like(fin)
            Q.pack_fermions(fin.data_ptr(), None, [x.data_ptr() for x in src], Q.QCU_SRC_EO_HALF, 1 - parity, prec)
            Q.dslash_mrhs(fref.data_ptr(), None, fin.data_ptr(), None, nrhs, parity, dagger, prec)
            Q.synchronize()
            gc, g12 = coalesced_gauge(torch, g, prec)
            fout = torch.full_like(fin, float("nan"))
            segs.append({"lattice": L, "gauge": gc.data_ptr(), "gauge_two_row": g12.data_ptr(), "in_": fin.data_ptr(),
                         "out": fout.data_ptr(), "nrhs": nrhs, "parity": parity, "dagger": dagger,
                         "antiperiodic_t": True})
            keep += [gc, g12, fin]
            refs.append((fref[: db // 8], fout[: db // 8]))  # the field, without the slack words
            data.append((L, g, psi, parity, dagger, nrhs))
        Q.dslash_segments(segs, 3, prec)
        Q.synchronize()
        for k, (fref, fout) in enumerate(refs):
            assert torch.equal(fout, fref), k  # bitwise, the per-lattice launch's result
        # and the oracle, through the caller layout
        for k, (L, g, psi, parity, dagger, nrhs) in enumerate(data):
            Q.initGridSize(L, 3)
            outs = [torch.zeros((S.half_volume(L), 4, 3), dtype=torch.complex128, device="cuda") for _ in range(nrhs)]
            Q.unpack_fermions([o.data_ptr() for o in outs], refs[k][1].data_ptr(), None, Q.QCU_SRC_EO_HALF, parity,
                              prec)
            Q.synchronize()
            got = np.stack([o.cpu().numpy() for o in outs])
            assert rel(got, O.dslash(psi, g, L, parity, dagger, True)) < TOL[prec], k
    finally:
        os.environ.pop("QCU_DSLASH_CONFIG", None)


def test_work_list_fallback_for_odd_rhs(cuda, qcu_lib):
    """nrhs = 3 does not fit R = 2: the segments run one launch each and are
    still correct; xpay coefficients are applied per segment."""
    torch, Q = cuda, qcu_lib
    os.environ["QCU_DSLASH_CONFIG"] = "2,64,2,1,0,0,0,1"
    try:
        segs, checks, keep = [], [], []
        for k, (L, nrhs) in enumerate([((4, 4, 4, 8), 3), ((8, 4, 4, 4), 4)]):
            g = S.random_gauge(L, 3, seed=930 + k)
            psi = S.random_fermions(L, 3, nrhs, seed=931 + k)
            xin = S.random_fermions(L, 3, nrhs, seed=932 + k)
            Q.initGridSize(L, 3)
            src = [dev(torch, psi[r]) for r in range(nrhs)]
            xs = [dev(torch, xin[r]) for r in range(nrhs)]
            db, _ = Q.field_bytes(1, nrhs)
            fin, fx, fout = (torch.zeros(db // 8 + 2, dtype=torch.float64, device="cuda") for _ in range(3))
            Q.pack_fermions(fin.data_ptr(), None, [x.data_ptr() for x in src], Q.QCU_SRC_EO_HALF, 1, 1)
            Q.pack_fermions(fx.data_ptr(), None, [x.data_ptr() for x in xs], Q.QCU_SRC_EO_HALF, 0, 1)
            gc, g12 = coalesced_gauge(torch, g, 1)
            segs.append({"lattice": L, "gauge": gc.data_ptr(), "gauge_two_row": g12.data_ptr(), "in_": fin.data_ptr(),
                         "out": fout.data_ptr(), "x": fx.data_ptr(), "a": 0.5, "b": -2.0, "nrhs": nrhs, "parity": 0,
                         "dagger": 0, "antiperiodic_t": False})
            keep += [gc, g12, fin, fx]
            checks.append((L, g, psi, xin, nrhs, fout))
        Q.dslash_segments(segs, 3, 1)
        Q.synchronize()
        for L, g, psi, xin, nrhs, fout in checks:
            Q.initGridSize(L, 3)
            outs = [torch.zeros((S.half_volume(L), 4, 3), dtype=torch.complex128, device="cuda") for _ in range(nrhs)]
            Q.unpack_fermions([o.data_ptr() for o in outs], fout.data_ptr(), None, Q.QCU_SRC_EO_HALF, 0, 1)
            Q.synchronize()
            got = np.stack([o.cpu().numpy() for o in outs])
            want = 0.5 * O.dslash(psi, g, L, 0, 0, False) - 2.0 * xin
            assert rel(got, want) < TOL[1]
    finally:
        os.environ.pop("QCU_DSLASH_CONFIG", None)
