"""GPU parity of the MRHS Wilson dslash through the C ABI (qcu.h), against
the FP64 oracle, the reference kernel's golden outputs and, when
oracle/_ref/ is present, the reference kernel itself on the same inputs.

Tolerances (relative L2): 1e-13 FP64, 1e-6 FP32, 5e-3 FP16/BF16 storage."""
import ctypes
import json
import os

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import TOL, abi_dslash, dev, rel

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("prec", [2, 1, 0, 4])
def test_config0_eo_oe_antiperiodic(cuda, qcu_lib, prec):
    """8^4 SU(3) nrhs=4, antiperiodic t: D_eo and D_oe once each, both dagger flags."""
    L = (8, 8, 8, 8)
    g = S.random_gauge(L, 3, seed=31)
    psi = S.random_fermions(L, 3, 4, seed=32)
    for parity in (0, 1):
        for dag in (0, 1):
            got = abi_dslash(cuda, qcu_lib, psi, g, L, parity, dag, prec, antiperiodic_t=True)
            ref = O.dslash(psi, g, L, parity, dag, True)
            assert rel(got, ref) < TOL[prec], (parity, dag)


def test_golden_reference_outputs(cuda, qcu_lib):
    """Against the reference kernel's stored outputs (bitwise-identical inputs)."""
    m = json.load(open(os.path.join(GOLDEN, "manifest.json")))
    case = [c for c in m["cases"] if c["name"] == "su3_d_4x4x4x8_full"][0]
    data = np.load(os.path.join(GOLDEN, case["file"]))
    for c in case["combos"]:
        got = abi_dslash(cuda, qcu_lib, data["psi"], data["gauge"], tuple(case["L"]), c["parity"], c["dagger"], 2,
                         c["antiperiodic_t"])
        assert rel(got, data[c["key"]]) < 1e-13


@pytest.mark.parametrize("n,nrhs", [(3, 1), (3, 2), (3, 3), (3, 5), (3, 12), (3, 24), (4, 2), (4, 16), (5, 1),
                                    (6, 2), (7, 1), (8, 2), (8, 4)])
@pytest.mark.parametrize("prec", [2, 1])
def test_colours_and_rhs_counts(cuda, qcu_lib, n, nrhs, prec):
    L = (4, 4, 4, 4)
    g = S.random_gauge(L, n, seed=40 + n)
    psi = S.random_fermions(L, n, nrhs, seed=50 + nrhs)
    got = abi_dslash(cuda, qcu_lib, psi, g, L, 1, 0, prec, antiperiodic_t=True)
    assert rel(got, O.dslash(psi, g, L, 1, 0, True)) < TOL[prec]


@pytest.mark.parametrize("prec", [2, 1, 0, 4])
@pytest.mark.parametrize("n", [3, 4, 6, 8])
@pytest.mark.parametrize("L", [(4, 4, 4, 8), (12, 4, 6, 4)])
def test_every_kernel_shape(cuda, qcu_lib, prec, n, L):
    """Every compiled shape, pinned in turn, against the oracle: register
    kernels (R, register cap, packed, two-row links, links staged by TMA),
    TMA-staged kernels (R, stages) and the tensor-core kernel (BF16, N >= 4).
    The packed FP32x2 kernels (links from L1 or from shared memory) and the
    staged kernels are bit-identical to the scalar register kernel of the
    same R and link form (they perform its FMA sequence); the
    tensor-core kernel rounds its operands to BF16 and meets the 16-bit
    tolerance."""
    Q = qcu_lib
    nrhs = 12
    g = S.random_gauge(L, n, seed=70 + n)
    psi = S.random_fermions(L, n, nrhs, seed=71)
    ref = {d: O.dslash(psi, g, L, d, d, True) for d in (0, 1)}
    shapes = Q.dslash_kernels(prec, n)
    assert shapes
    outs = {}
    try:
        for i, (R, minb, pk, st, rc, lt) in enumerate(shapes):
            if nrhs % R or (n >= 6 and st != 0):  # N >= 6: staged and tensor-core kernels in their own tests
                continue
            os.environ["QCU_DSLASH_CONFIG"] = ("1,0,0,0,0,0,%d" % -st if st < 0 else "%d,%d,%d,%d,%d,0,0,%d,%d" % (
                R, (32, 64, 128, 256)[i % 4], minb, pk, st, rc, lt))
            for d in (0, 1):  # (parity 0, dagger 0) and (parity 1, dagger 1)
                got = abi_dslash(cuda, Q, psi, g, L, d, d, prec, antiperiodic_t=True)
                assert rel(got, ref[d]) < TOL[prec], (R, minb, pk, st, rc, lt, d)
                outs[(R, minb, pk, st, rc, lt, d)] = got
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]
    for (R, minb, pk, st, rc, lt, d), got in outs.items():
        if pk or st > 0:
            for (r2, m2, p2, s2, rc2, lt2, d2), other in outs.items():
                if r2 == R and d2 == d and not p2 and not s2 and rc2 == rc:
                    assert np.array_equal(got, other), (R, minb, pk, st, rc, lt, m2, d)


@pytest.mark.parametrize("prec", [2, 1, 4])
def test_reconstructed_links_only_for_su3_fields(cuda, qcu_lib, prec):
    """The two-row (reconstruct-12) kernels: exact against the oracle on an
    SU(3) field; on a field that is not SU(3) (links scaled by 1.01) the
    library keeps the full links, so the result is still the oracle's."""
    Q = qcu_lib
    L, nrhs = (4, 4, 4, 8), 4
    g = S.random_gauge(L, 3, seed=97)
    psi = S.random_fermions(L, 3, nrhs, seed=98)
    R = 1 if prec == 2 else 2
    minb = 1 if prec != 4 else 2
    os.environ["QCU_DSLASH_CONFIG"] = "%d,64,%d,0,0,0,0,1" % (R, minb)
    try:
        for gauge in (g, 1.01 * g):
            got = abi_dslash(cuda, Q, psi, gauge, L, 1, 0, prec, antiperiodic_t=True)
            assert rel(got, O.dslash(psi, gauge, L, 1, 0, True)) < TOL[prec]
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]


def _pin(R, minb, pk, rc, lt, block=64):
    return "%d,%d,%d,%d,0,0,0,%d,%d" % (R, block, minb, pk, rc, lt)


@pytest.mark.parametrize("prec,rc,L,nrhs", [
    (1, 1, (4, 4, 4, 8), 12), (1, 0, (4, 4, 4, 8), 2), (1, 0, (12, 4, 6, 4), 12), (1, 1, (16, 6, 4, 10), 64),
    (1, 0, (8, 8, 8, 16), 24), (1, 1, (8, 8, 8, 16), 4), (4, 1, (8, 8, 8, 16), 12), (4, 1, (16, 6, 4, 10), 64),
    (1, 1, (32, 4, 2, 4), 12), (4, 1, (8, 4, 4, 4), 4)])
def test_link_staged_kernel(cuda, qcu_lib, prec, rc, L, nrhs):
    """The register kernel with its links staged by TMA into shared memory
    (one CTA per x-row, eight boxes on eight mbarriers): against the oracle on
    both parities, dagger flags and antiperiodic t, for rows of 2..16 sites,
    1..32 RHS groups, full and two-row links, FP32 and BF16 storage; launched
    (not a fallback) and bit-identical to the register kernel of the same R
    and link form."""
    Q = qcu_lib
    g = S.random_gauge(L, 3, seed=600 + nrhs)
    psi = S.random_fermions(L, 3, nrhs, seed=601 + nrhs)
    minb = [s[1] for s in Q.dslash_kernels(prec, 3) if s[0] == 2 and s[2] == 1 and s[4] == rc and s[5] == 1][0]
    plain = [s[1] for s in Q.dslash_kernels(prec, 3) if s[0] == 2 and s[2] == 1 and s[4] == rc and s[5] == 0]
    try:
        for d in (0, 1):
            os.environ["QCU_DSLASH_CONFIG"] = _pin(2, minb, 1, rc, 1)
            got = abi_dslash(cuda, Q, psi, g, L, d, d, prec, antiperiodic_t=True)
            assert Q.last_dslash_shape()[4:] == (rc, 1), Q.last_dslash_shape()
            assert rel(got, O.dslash(psi, g, L, d, d, True)) < TOL[prec], d
            os.environ["QCU_DSLASH_CONFIG"] = _pin(2, plain[0], 1, rc, 0)
            other = abi_dslash(cuda, Q, psi, g, L, d, d, prec, antiperiodic_t=True)
            assert Q.last_dslash_shape()[5] == 0
            assert np.array_equal(got, other), d
    finally:
        os.environ.pop("QCU_DSLASH_CONFIG", None)


@pytest.mark.parametrize("L,prec,rc", [((6, 4, 4, 4), 1, 0), ((6, 4, 4, 4), 4, 1), ((10, 4, 2, 4), 4, 1),
                                       ((12, 4, 6, 4), 1, 1)])
def test_link_staged_kernel_falls_back(cuda, qcu_lib, L, prec, rc):
    """Rows the link-staged kernel cannot copy as a TMA box: component rows
    that are not a whole number of 16-byte units (X/2 = 3 FP32 sites, 24
    bytes; 3 or 5 BF16 sites), and two-row links of rows that do not divide
    the gauge's groups of 32 sites (X/2 = 6).  The pinned link-staged shape
    runs the register kernel, with the oracle's result."""
    Q = qcu_lib
    g = S.random_gauge(L, 3, seed=610)
    psi = S.random_fermions(L, 3, 4, seed=611)
    minb = [s[1] for s in Q.dslash_kernels(prec, 3) if s[0] == 2 and s[2] == 1 and s[4] == rc and s[5] == 1][0]
    os.environ["QCU_DSLASH_CONFIG"] = _pin(2, minb, 1, rc, 1)
    try:
        got = abi_dslash(cuda, Q, psi, g, L, 1, 0, prec, antiperiodic_t=True)
        assert Q.last_dslash_shape()[5] == 0
        assert rel(got, O.dslash(psi, g, L, 1, 0, True)) < TOL[prec]
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]


def test_link_staged_kernel_in_masked_solve(cuda, qcu_lib):
    """The link-staged kernel as the FP32 inner dslash of the masked eo-CG
    (8^3 x 16 SU(3), 6 RHS, one zero source, one 1e-3 smaller so that RHS
    converge at different iterations): every RHS meets the tolerance by the
    oracle's FP64 true residual and the zero source gives zero."""
    torch, Q = cuda, qcu_lib
    L, n, nr, kappa, tol = (8, 8, 8, 16), 3, 6, 0.12, 1e-9
    g = S.random_gauge(L, n, seed=620)
    b = S.random_fermions(L, n, nr, seed=621, parities=2)
    b[1] *= 1e-3
    b[4] = 0
    minb = [s[1] for s in Q.dslash_kernels(1, 3) if s[0] == 2 and s[2] == 1 and s[4] == 1 and s[5] == 1][0]
    os.environ["QCU_DSLASH_CONFIG"] = _pin(2, minb, 1, 1, 1)
    try:
        Q.initGridSize(L, n)
        Q.set_antiperiodic_t(True)
        dg = dev(torch, g)
        Q.loadQcuGauge(dg.data_ptr())
        db = [dev(torch, b[r]) for r in range(nr)]
        dx = [torch.zeros_like(x) for x in db]
        p = Q.solver_params(kappa=kappa, tol=tol, inner_precision=1, max_iter=5000)
        Q.invert([x.data_ptr() for x in dx], [x.data_ptr() for x in db], p)
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]
    assert float(dx[4].abs().max()) == 0.0
    for r in range(nr):
        assert p.converged[r], r
        if r != 4:
            res = O.true_residual(dx[r].cpu().numpy(), b[r], g, L, kappa, antiperiodic_t=True)
            assert res < 2 * tol, (r, res)


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("n,nrhs", [(4, 16), (8, 16), (6, 24), (8, 64), (5, 128), (3, 32), (7, 36), (8, 8)])
def test_tensor_core_kernel(cuda, qcu_lib, n, nrhs, variant):
    """The tcgen05 kernels (BF16 storage and operands, FP32 accumulation in
    tensor memory) against the FP64 oracle: both parities and dagger flags,
    antiperiodic t, RHS counts that fill the 128 MMA rows, leave them partly
    empty, take two tiles, or end inside the second 32-RHS box.  Variants 1-3
    are the projected half-spinor kernel (N >= 4; the TMA ring for N = 4, 6,
    8), 4-6 the spinor-operand kernel with 4-6 ring stages, 7-8 the same with
    deeper rings of one 32-RHS half per stage (launched for tiles of at most
    32 RHS; larger tiles run another kernel)."""
    L = (4, 4, 4, 8)
    g = S.random_gauge(L, n, seed=90 + n)
    psi = S.random_fermions(L, n, nrhs, seed=91)
    if variant <= 3 and n == 3:
        pytest.skip("the projected kernel is compiled for N >= 4")
    if variant in (2, 3) and n in (5, 7):
        pytest.skip("the projected kernel's TMA ring is compiled for N = 4, 6, 8")
    os.environ["QCU_DSLASH_CONFIG"] = "1,0,0,0,0,0,%d" % variant
    try:
        tile = max(t for t in range(4, 65, 4) if nrhs % t == 0)  # RHS per tile of the spinor-operand kernel
        for parity, dag in ((0, 0), (1, 1), (1, 0)):
            got = abi_dslash(cuda, qcu_lib, psi, g, L, parity, dag, 4, antiperiodic_t=True)
            assert rel(got, O.dslash(psi, g, L, parity, dag, True)) < TOL[4], (parity, dag)
            if variant >= 4 and (variant <= 6 or tile <= 32):
                assert qcu_lib.last_dslash_shape()[3] == -variant
        assert qcu_lib.tune_dslash(nrhs, 4)[4] == -variant  # the pinned shape is this tensor-core variant
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]


@pytest.mark.parametrize("variant", [1, 4])
def test_tensor_core_xpay_resident(cuda, qcu_lib, variant):
    """xpay epilogue of the tensor-core kernels on resident BF16 fields."""
    torch, Q = cuda, qcu_lib
    L, n, nrhs = (4, 4, 4, 8), 4, 16
    g = S.random_gauge(L, n, seed=95)
    full = S.random_fermions(L, n, nrhs, seed=96, parities=2)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(False)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    db, nb = Q.field_bytes(4, nrhs)
    bufs = [torch.empty(db // 8 + 2, dtype=torch.float64, device="cuda") for _ in range(3)]
    norms = [torch.empty(nb // 4 + 4, dtype=torch.float32, device="cuda") for _ in range(3)]
    src = [dev(torch, full[r]) for r in range(nrhs)]
    ptrs = [x.data_ptr() for x in src]
    Q.pack_fermions(bufs[0].data_ptr(), norms[0].data_ptr(), ptrs, Q.QCU_SRC_EO_FULL, 0, 4)
    Q.pack_fermions(bufs[1].data_ptr(), norms[1].data_ptr(), ptrs, Q.QCU_SRC_EO_FULL, 1, 4)
    a, b = 0.37, -1.25
    os.environ["QCU_DSLASH_CONFIG"] = "1,0,0,0,0,0,%d" % variant
    try:
        Q.dslash_xpay_mrhs(bufs[2].data_ptr(), norms[2].data_ptr(), bufs[0].data_ptr(), norms[0].data_ptr(),
                           bufs[1].data_ptr(), norms[1].data_ptr(), nrhs, 1, 0, 4, a, b)
        outs = [torch.zeros((S.half_volume(L), 4, n), dtype=torch.complex128, device="cuda") for _ in range(nrhs)]
        Q.unpack_fermions([o.data_ptr() for o in outs], bufs[2].data_ptr(), norms[2].data_ptr(),
                          Q.QCU_SRC_EO_HALF, 1, 4)
        Q.synchronize()
    finally:
        del os.environ["QCU_DSLASH_CONFIG"]
    got = np.stack([o.cpu().numpy() for o in outs])
    want = a * O.dslash(full[:, 0], g, L, 1, 0, False) + b * full[:, 1]
    assert rel(got, want) < TOL[4]


@pytest.mark.parametrize("prec", [0, 4])
@pytest.mark.parametrize("n,nrhs", [(3, 4), (3, 12), (4, 8), (8, 2)])
def test_half_storage(cuda, qcu_lib, prec, n, nrhs):
    L = (4, 4, 4, 8)
    g = S.random_gauge(L, n, seed=60 + n)
    psi = S.random_fermions(L, n, nrhs, seed=61)
    got = abi_dslash(cuda, qcu_lib, psi, g, L, 0, 1, prec)
    assert rel(got, O.dslash(psi, g, L, 0, 1)) < TOL[prec]


@pytest.mark.parametrize("L", [(6, 4, 4, 4), (2, 2, 2, 2), (4, 6, 2, 10), (12, 2, 4, 6)])
def test_odd_and_tiny_lattices(cuda, qcu_lib, L):
    """Half volumes that are not multiples of the block size (the reference
    kernel has no tail guard) and odd half-X extents."""
    g = S.random_gauge(L, 3, seed=70)
    psi = S.random_fermions(L, 3, 3, seed=71)
    for prec in (2, 1):
        got = abi_dslash(cuda, qcu_lib, psi, g, L, 0, 0, prec, antiperiodic_t=True)
        assert rel(got, O.dslash(psi, g, L, 0, 0, True)) < TOL[prec]


def test_against_reference_kernel_same_inputs(cuda, qcu_lib):
    from oracle import ref_runner
    ref_runner.require(pytest)
    ref = ref_runner.RefModule()
    # every instantiation of the reference module (ref_runner.DSLASH_VARIANTS) at least once
    for L, n, nrhs, prec in [((8, 8, 8, 8), 3, 4, "d"), ((8, 4, 4, 8), 3, 5, "d"), ((4, 4, 4, 8), 4, 2, "d"),
                             ((8, 8, 8, 8), 3, 4, "f"), ((4, 4, 4, 8), 5, 1, "f"), ((8, 4, 4, 8), 3, 1, "d"),
                             ((4, 8, 4, 8), 3, 2, "d"), ((4, 4, 8, 8), 3, 3, "d"), ((8, 4, 4, 8), 3, 1, "f"),
                             ((4, 4, 4, 8), 4, 2, "f"), ((4, 4, 4, 8), 5, 1, "d")]:
        g = S.random_gauge(L, n, seed=80)
        psi = S.random_fermions(L, n, nrhs, seed=81)
        for parity, dag, ap in [(0, 0, False), (1, 1, True)]:
            r = ref.dslash(psi, g, L, parity, dag, prec, ap)
            ours = abi_dslash(cuda, qcu_lib, psi, g, L, parity, dag, 2 if prec == "d" else 1, ap)
            assert rel(ours, r) < (1e-13 if prec == "d" else 2e-6)


def test_mrhs_equals_single_rhs(cuda, qcu_lib):
    """Batching is exact: the 12-RHS result equals 12 one-RHS calls bitwise (FP64)."""
    L = (8, 4, 4, 8)
    g = S.random_gauge(L, 3, seed=90)
    psi = S.random_fermions(L, 3, 12, seed=91)
    batch = abi_dslash(cuda, qcu_lib, psi, g, L, 1, 0, 2)
    for r in (0, 5, 11):
        one = abi_dslash(cuda, qcu_lib, psi[r:r + 1], g, L, 1, 0, 2)
        assert np.array_equal(one[0], batch[r])


@pytest.mark.parametrize("prec", [2, 1, 0, 4])
def test_resident_mrhs_api_and_xpay(cuda, qcu_lib, prec):
    """qcuPackFermions -> qcuDslashXpayMRHS -> qcuUnpackFermions, lexicographic input."""
    torch, Q = cuda, qcu_lib
    L = (4, 4, 4, 8)
    n, nrhs = 3, 6
    g = S.random_gauge(L, n, seed=100)
    full = S.random_fermions(L, n, nrhs, seed=101, parities=2)       # (nrhs, 2, Vh, 4, n)
    lex = np.stack([O.eo_to_lex(full[r], L) for r in range(nrhs)])  # (nrhs, V, 4, n)
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(True)
    dg = dev(torch, g)
    Q.loadQcuGauge(dg.data_ptr())
    db, nb = Q.field_bytes(prec, nrhs)
    bufs = [torch.empty(db // 8 + 2, dtype=torch.float64, device="cuda") for _ in range(3)]
    norms = [torch.empty(max(nb, 16) // 4, dtype=torch.float32, device="cuda") for _ in range(3)]
    nrm = (lambda i: norms[i].data_ptr()) if nb else (lambda i: None)
    src = [dev(torch, lex[r]) for r in range(nrhs)]
    ptrs = [s.data_ptr() for s in src]
    Q.pack_fermions(bufs[0].data_ptr(), nrm(0), ptrs, Q.QCU_SRC_LEX, 1, prec)  # odd input
    Q.pack_fermions(bufs[1].data_ptr(), nrm(1), ptrs, Q.QCU_SRC_LEX, 0, prec)  # even x
    a, b = -0.0144, 1.0
    Q.dslash_xpay_mrhs(bufs[2].data_ptr(), nrm(2), bufs[0].data_ptr(), nrm(0), bufs[1].data_ptr(), nrm(1), nrhs, 0, 0,
                       prec, a, b)
    outs = [torch.zeros((S.half_volume(L), 4, n), dtype=torch.complex128, device="cuda") for _ in range(nrhs)]
    Q.unpack_fermions([o.data_ptr() for o in outs], bufs[2].data_ptr(), nrm(2), Q.QCU_SRC_EO_HALF, 0, prec)
    Q.synchronize()
    got = np.stack([o.cpu().numpy() for o in outs])
    want = a * O.dslash(full[:, 1], g, L, 0, 0, True) + b * full[:, 0]
    assert rel(got, want) < TOL[prec]


def test_layout_lex_eo_and_lex_gauge(cuda, qcu_lib):
    torch, Q = cuda, qcu_lib
    L = (4, 2, 6, 4)
    n = 3
    g = S.random_gauge(L, n, seed=110)
    psi = S.random_fermions(L, n, 2, seed=111)
    # gauge given lexicographically: [4][V][N][N]
    V = 2 * S.half_volume(L)
    glex = np.stack([O.eo_to_lex(g[mu], L) for mu in range(4)])
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(False)
    dgl = dev(torch, glex)
    Q.load_gauge_lex(dgl.data_ptr())
    Q.getDslash(0, 0.0, n, 2, 2)
    ins = [dev(torch, psi[r]) for r in range(2)]
    outs = [torch.zeros_like(x) for x in ins]
    for r in range(2):
        Q.pushBackFermions(outs[r].data_ptr(), ins[r].data_ptr())
    Q.startDslash(0, 0)
    got = np.stack([o.cpu().numpy() for o in outs])
    assert rel(got, O.dslash(psi, g, L, 0, 0)) < 1e-13
    # fermion lex <-> eo
    rng = np.random.default_rng(112)
    lex = rng.standard_normal((V, 4, n)) + 1j * rng.standard_normal((V, 4, n))
    dl = dev(torch, lex)
    de = torch.zeros((2, V // 2, 4, n), dtype=torch.complex128, device="cuda")
    Q.lex_to_eo(de.data_ptr(), dl.data_ptr(), 4 * n)
    assert np.array_equal(de.cpu().numpy(), O.lex_to_eo(lex, L))
    dl2 = torch.zeros_like(dl)
    Q.eo_to_lex(dl2.data_ptr(), de.data_ptr(), 4 * n)
    assert np.array_equal(dl2.cpu().numpy(), lex)


def test_deprecated_entry_points(cuda, qcu_lib):
    """dslashQcu / fullDslashQcu (no-op stubs in the reference) compute the hop."""
    torch, Q = cuda, qcu_lib
    L = (4, 4, 4, 4)
    g = S.random_gauge(L, 3, seed=120)
    full = S.random_fermions(L, 3, 1, seed=121, parities=2)[0]
    Q.set_antiperiodic_t(False)
    dg, din = dev(torch, g), dev(torch, full)
    dout = torch.zeros_like(din)
    Q.fullDslashQcu(dout.data_ptr(), din.data_ptr(), dg.data_ptr(), L, 1)
    got = dout.cpu().numpy()
    for p in (0, 1):
        assert rel(got[p], O.dslash(full[1 - p][None], g, L, p, 1)[0]) < 1e-13
    half_in = dev(torch, full[1])
    half_out = torch.zeros_like(half_in)
    Q.dslashQcu(half_out.data_ptr(), half_in.data_ptr(), dg.data_ptr(), L, 0)
    assert rel(half_out.cpu().numpy(), O.dslash(full[1][None], g, L, 0, 0)[0]) < 1e-13


def test_cxx_storage_api(cuda, qcu_lib):
    """qcu::storage::shiftVectorStorage / shiftGaugeStorage (reference C++ API)."""
    torch, Q = cuda, qcu_lib
    lib = Q.lib()
    L = (4, 4, 4, 8)
    vh = S.half_volume(L)
    psi = S.random_fermions(L, 3, 1, seed=130)[0]
    g = S.random_gauge(L, 3, seed=131)
    fv = getattr(lib, Q.CXX_SYMBOLS[0])
    fg = getattr(lib, Q.CXX_SYMBOLS[1])
    for f in (fv, fg):
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_int] * 4
        f.restype = None
    src = dev(torch, psi)
    dst = torch.zeros((12, vh), dtype=torch.complex128, device="cuda")
    fv(dst.data_ptr(), src.data_ptr(), 0, L[0] // 2, L[1], L[2], L[3])
    assert np.array_equal(dst.cpu().numpy(), psi.reshape(vh, 12).T)
    back = torch.zeros_like(src)
    fv(back.data_ptr(), dst.data_ptr(), 1, L[0] // 2, L[1], L[2], L[3])
    assert np.array_equal(back.cpu().numpy(), psi)
    gs = dev(torch, g)
    gd = torch.zeros((4, 2, 9, vh), dtype=torch.complex128, device="cuda")
    fg(gd.data_ptr(), gs.data_ptr(), 0, *L)
    assert np.array_equal(gd.cpu().numpy(), g.reshape(4, 2, vh, 9).transpose(0, 1, 3, 2))


def test_full_size_fp32_against_oracle(cuda, qcu_lib):
    """32^3 x 64, SU(3), nrhs = 12 in FP32 (the benchmark workload): two RHS
    checked against the oracle, all twelve by linearity across RHS."""
    torch, Q = cuda, qcu_lib
    L = (32, 32, 32, 64)
    g = S.random_gauge(L, 3, seed=140)
    rng = np.random.default_rng(141)
    vh = S.half_volume(L)
    base = (rng.standard_normal((2, vh, 4, 3)) + 1j * rng.standard_normal((2, vh, 4, 3))) * np.sqrt(0.5)
    coef = rng.standard_normal((12, 2))
    psi = np.einsum("rk,kvsa->rvsa", coef, base)  # every RHS a combination of the two bases
    got = abi_dslash(torch, Q, psi, g, L, 1, 0, 1, antiperiodic_t=True)
    ref = O.dslash(base, g, L, 1, 0, True)
    want = np.einsum("rk,kvsa->rvsa", coef, ref)
    for r in range(12):
        assert rel(got[r], want[r]) < 1e-6


def test_queue_batches_and_argument_edges(cuda, qcu_lib):
    """startDslash with more RHS than one launch takes (300: a batch of 256,
    then one of 44) against the oracle; a second startDslash on the emptied
    queue is a no-op; resident calls with no RHS, a null or in-place output or
    a misaligned field are rejected with QCU_ERR_INVALID_ARGUMENT before any
    GPU work."""
    Q = qcu_lib
    L, n, nrhs = (4, 4, 4, 8), 3, 300
    g = S.random_gauge(L, n, seed=111)
    psi = S.random_fermions(L, n, nrhs, seed=112)
    got = abi_dslash(cuda, Q, psi, g, L, 1, 0, 1, antiperiodic_t=True)
    assert rel(got, O.dslash(psi, g, L, 1, 0, True)) < TOL[1]
    Q.clear_error()
    Q.startDslash(0, 0)
    assert Q.last_error()[0] == 0
    db, _ = Q.field_bytes(1, 4)
    a = cuda.zeros(db // 8 + 2, dtype=cuda.float64, device="cuda")
    b = cuda.zeros_like(a)
    for args in ((b.data_ptr(), None, a.data_ptr(), None, 0, 0, 0, 1),
                 (0, None, a.data_ptr(), None, 4, 0, 0, 1),
                 (a.data_ptr(), None, a.data_ptr(), None, 4, 0, 0, 1),
                 (b.data_ptr() + 8, None, a.data_ptr(), None, 4, 0, 0, 1)):
        with pytest.raises(Q.QcuError) as e:
            Q.dslash_mrhs(*args)
        assert e.value.code == 2, args
    Q.clear_error()
