"""Rate of this library's MRHS dslash against the reference's own GPU kernel
(include/kernels/wilson_dslash_4d.cuh, rebuilt for sm_103a by
oracle/build_ref.sh and launched through oracle/ref_runner.py), on the same
GPU and the same 32^3x64 SU(3) inputs.

Both sides apply D_eo once to device-resident fields in their own layouts
(the reference: one [4N][Vh] array per RHS; this library: the resident MRHS
field), timed with CUDA events after a warm-up.  The reference instantiates
at most 4 RHS in FP32 and 5 in FP64 per launch, so the comparison runs at
nrhs = 4.  The rates are printed (pytest -s), and this library must be at
least as fast as the kernel it replaces."""
import ctypes

import pytest

from mrhs_qcu_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _ms_per_call(torch, fn, reps=10):
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


@pytest.mark.parametrize("prec", ["f", "d"])
def test_rate_against_reference_kernel(cuda, qcu_lib, prec):
    from oracle import ref_runner
    ref_runner.require(pytest)
    torch, Q = cuda, qcu_lib
    L, n, nrhs = (32, 32, 32, 64), 3, 4
    vh = S.half_volume(L)
    gen = torch.Generator(device="cuda").manual_seed(5)
    g = S.random_sun_torch(4 * 2 * vh, n, gen).view(4, 2, vh, n, n)
    psi = torch.complex(torch.randn((nrhs, vh, 4, n), generator=gen, device="cuda", dtype=torch.float64),
                        torch.randn((nrhs, vh, 4, n), generator=gen, device="cuda", dtype=torch.float64))

    # the reference kernel on its coalesced layouts (ref_runner.dslash, without the host round trips)
    ref = ref_runner.RefModule()
    cdt = torch.complex128 if prec == "d" else torch.complex64
    g_soa = g.reshape(4, 2, vh, n * n).permute(0, 1, 3, 2).contiguous().to(cdt)
    ins = [psi[r].reshape(vh, 4 * n).t().contiguous().to(cdt) for r in range(nrhs)]
    outs = [torch.zeros((4 * n, vh), dtype=cdt, device="cuda") for _ in range(nrhs)]

    class Mrhs(ctypes.Structure):
        _fields_ = [("fermion", ctypes.c_void_p * nrhs)]

    o, i = Mrhs(), Mrhs()
    for r in range(nrhs):
        o.fermion[r] = outs[r].data_ptr()
        i.fermion[r] = ins[r].data_ptr()
    flag = (ctypes.c_double if prec == "d" else ctypes.c_float)(1.0)
    name = "qcuref_dslash_%s_%d_%d" % (prec, n, nrhs)
    args = [o, i, ctypes.c_void_p(g_soa.data_ptr()), flag] + [ctypes.c_int(x) for x in L] + [ctypes.c_int(0)]
    ms_ref = _ms_per_call(torch, lambda: ref.launch(name, (vh + 255) // 256, 256, args))

    # this library: resident MRHS field, autotuned kernel
    qp = 2 if prec == "d" else 1
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(False)
    Q.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        Q.loadQcuGauge(g.data_ptr())
        Q.getDslash(Q.DSLASH_WILSON, 0.0, n, nrhs, qp)
        db, _ = Q.field_bytes(qp, nrhs)
        fin = torch.empty(db // 8 + 2, dtype=torch.float64, device="cuda")
        fout = torch.empty_like(fin)
        Q.pack_fermions(fin.data_ptr(), None, [psi[r].data_ptr() for r in range(nrhs)], Q.QCU_SRC_EO_HALF, 1, qp)
        Q.tune_dslash(nrhs, qp)
        ms_ours = _ms_per_call(torch, lambda: Q.dslash_mrhs(fout.data_ptr(), None, fin.data_ptr(), None, nrhs, 0, 0,
                                                             qp))
    finally:
        Q.set_stream(None)
    units = vh * nrhs
    print("\n%s SU(3) 32^3x64 nrhs %d: reference kernel %.3f ms (%.3f G site*RHS/s), this library %.3f ms "
          "(%.3f G site*RHS/s), %.2fx" % ("FP64" if prec == "d" else "FP32", nrhs, ms_ref, units / ms_ref / 1e6,
                                          ms_ours, units / ms_ours / 1e6, ms_ref / ms_ours))
    assert ms_ours <= ms_ref
