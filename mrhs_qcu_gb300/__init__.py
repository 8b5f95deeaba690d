"""mrhs_qcu_gb300 -- GB300 (sm_103a) multi-right-hand-side even-odd Wilson
dslash, layout transforms and even-odd preconditioned Krylov solves behind
the reference's ``qcu.h`` C ABI.

The compute path is ``libqcu.so`` (CUDA kernels + C++ host layer, built
in-tree by ``mrhs_qcu_gb300.build``).  This module is a thin ctypes mirror of
the C ABI with the reference's function names (include/qcu.h:19-30 of the
reference) plus the extensions of ``include/qcu_gb300.h``.  There is no CPU
fallback: importing fails if the library has not been built.

Pointers are device addresses (ints), e.g. ``tensor.data_ptr()`` of a CUDA
tensor of dtype complex128 in the caller layouts documented in qcu.h.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libqcu.so")

# enum values of the reference (include/qcu_enum.h:4-12) + BF16 extension
QCU_HALF_PRECISION = 0
QCU_SINGLE_PRECISION = 1
QCU_DOUBLE_PRECISION = 2
QCU_BF16_PRECISION = 4
QCU_BF16_SITE_PRECISION = 5  # BF16, site-major field layout (tensor-core dslash)
EVEN_PARITY = 0
ODD_PARITY = 1
QCU_DAGGER_NO = 0
QCU_DAGGER_YES = 1
DSLASH_WILSON = 0
DSLASH_CLOVER = 1

QCU_SRC_EO_HALF = 0
QCU_SRC_EO_FULL = 1
QCU_SRC_LEX = 2
QCU_SOLVER_CG = 0
QCU_SOLVER_BICGSTAB = 1

STATUS = {0: "QCU_OK", 1: "QCU_ERR_NOT_INITIALIZED", 2: "QCU_ERR_INVALID_ARGUMENT", 3: "QCU_ERR_UNSUPPORTED",
          4: "QCU_ERR_CUDA", 5: "QCU_ERR_NO_GAUGE", 6: "QCU_ERR_NO_OPERATOR", 7: "QCU_ERR_NOT_CONVERGED",
          8: "QCU_ERR_BREAKDOWN", 9: "QCU_ERR_DEVICE_TIMEOUT", 10: "QCU_ERR_OUT_OF_MEMORY",
          11: "QCU_ERR_CAPACITY"}


class QcuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg.strip()))
        self.code = code


class QcuParam(ctypes.Structure):
    """include/qcu.h:7-9 of the reference."""
    _fields_ = [("lattice_size", ctypes.c_int * 4)]


class QcuGrid(ctypes.Structure):
    """include/qcu.h:11-15 of the reference."""
    _fields_ = [("grid_size", ctypes.c_int * 4)]


class QcuSolverParam(ctypes.Structure):
    _fields_ = [("solver", ctypes.c_int), ("inner_precision", ctypes.c_int), ("kappa", ctypes.c_double),
                ("tol", ctypes.c_double), ("max_iter", ctypes.c_int), ("delta", ctypes.c_double),
                ("use_graph", ctypes.c_int), ("src_mode", ctypes.c_int), ("use_clover", ctypes.c_int),
                ("iterations", ctypes.c_int),
                ("reliable_updates", ctypes.c_int), ("seconds", ctypes.c_double),
                ("true_residual", ctypes.c_double * 256), ("converged", ctypes.c_int * 256)]


# every symbol the public headers declare (include/qcu.h, include/qcu_gb300.h)
ABI_SYMBOLS = ["initGridSize", "pushBackFermions", "startDslash", "loadQcuGauge", "getDslash", "dslashQcu",
               "fullDslashQcu", "cg_inverter"]
EXT_SYMBOLS = ["qcuGetLastError", "qcuGetLastErrorString", "qcuClearError", "qcuVersion", "qcuSetAntiperiodicT",
               "qcuSetStream", "qcuSynchronize", "qcuFieldBytes", "qcuPackFermions", "qcuUnpackFermions",
               "qcuLoadGaugeLex", "qcuLexToEo", "qcuEoToLex", "qcuDslashMRHS", "qcuDslashXpayMRHS",
               "qcuTuneDslash", "qcuLastDslashShape", "qcuDslashKernels", "qcuMeasureFmaRate", "qcuSolverParamDefaults", "qcuInvert", "qcuNorm2MRHS",
               "qcuNorm2MRHSNoAlloc", "qcuBlasMRHS", "qcuCheckWaitTimeout", "qcuDslashSegments", "qcuLoadClover", "qcuCloverMRHS",
               "qcuServerCreate", "qcuServerAddGauge", "qcuServerSubmit", "qcuServerWait", "qcuServerStats",
               "qcuServerDestroy"]


class QcuHopSegment(ctypes.Structure):
    _fields_ = [("lattice", ctypes.c_int * 4), ("gauge", ctypes.c_void_p), ("gauge_two_row", ctypes.c_void_p),
                ("in_", ctypes.c_void_p), ("out", ctypes.c_void_p), ("x", ctypes.c_void_p),
                ("a", ctypes.c_double), ("b", ctypes.c_double), ("nrhs", ctypes.c_int), ("parity", ctypes.c_int),
                ("dagger", ctypes.c_int), ("antiperiodic_t", ctypes.c_int)]


class QcuRequestInfo(ctypes.Structure):
    _fields_ = [("done", ctypes.c_int), ("status", ctypes.c_int), ("nrhs", ctypes.c_int),
                ("iterations", ctypes.c_int), ("latency_s", ctypes.c_double), ("queue_s", ctypes.c_double),
                ("max_true_residual", ctypes.c_double), ("all_converged", ctypes.c_int)]


class QcuServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong), ("p50_s", ctypes.c_double),
                ("p99_s", ctypes.c_double), ("mean_s", ctypes.c_double), ("solves_per_s", ctypes.c_double),
                ("rhs_per_s", ctypes.c_double), ("hbm_used", ctypes.c_size_t)]
# C++ symbols with the reference's mangled names (include/qcu_storage.h)
CXX_SYMBOLS = ["_ZN3qcu7storage18shiftVectorStorageEPvS1_14ShiftDirectioniiii",
               "_ZN3qcu7storage17shiftGaugeStorageEPvS1_14ShiftDirectioniiii"]

_lib = None


def lib() -> ctypes.CDLL:
    """Load libqcu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libqcu.so is not built: run `python -m mrhs_qcu_gb300.build` "
                          "(or __graft_entry__.build()); there is no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    P, I, D, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
    PP = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "initGridSize": ([ctypes.POINTER(QcuGrid), ctypes.POINTER(QcuParam), I], None),
        "pushBackFermions": ([P, P], None),
        "startDslash": ([I, I], None),
        "loadQcuGauge": ([P], None),
        "getDslash": ([I, D, I, I, I], None),
        "dslashQcu": ([P, P, P, ctypes.POINTER(QcuParam), I], None),
        "fullDslashQcu": ([P, P, P, ctypes.POINTER(QcuParam), I], None),
        "cg_inverter": ([P, P, P, ctypes.POINTER(QcuParam), D, D], None),
        "qcuGetLastError": ([], I),
        "qcuGetLastErrorString": ([], ctypes.c_char_p),
        "qcuClearError": ([], None),
        "qcuVersion": ([], ctypes.c_char_p),
        "qcuSetAntiperiodicT": ([I], I),
        "qcuSetStream": ([P], I),
        "qcuSynchronize": ([], I),
        "qcuFieldBytes": ([I, I, ctypes.POINTER(S), ctypes.POINTER(S)], I),
        "qcuPackFermions": ([P, P, PP, I, I, I, I], I),
        "qcuUnpackFermions": ([PP, P, P, I, I, I, I], I),
        "qcuLoadGaugeLex": ([P], I),
        "qcuLexToEo": ([P, P, I], I),
        "qcuEoToLex": ([P, P, I], I),
        "qcuDslashMRHS": ([P, P, P, P, I, I, I, I], I),
        "qcuDslashXpayMRHS": ([P, P, P, P, P, P, I, I, I, I, D, D], I),
        "qcuTuneDslash": ([I, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I),
                           ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)], I),
        "qcuDslashKernels": ([I, I, ctypes.POINTER(I), I, ctypes.POINTER(I)], I),
        "qcuLastDslashShape": ([ctypes.POINTER(I)], I),
        "qcuMeasureFmaRate": ([I, ctypes.POINTER(ctypes.c_double)], I),
        "qcuLoadClover": ([P], I),
        "qcuCloverMRHS": ([P, P, P, P, I, I, I, I], I),
        "qcuSolverParamDefaults": ([ctypes.POINTER(QcuSolverParam)], None),
        "qcuInvert": ([PP, PP, I, ctypes.POINTER(QcuSolverParam)], I),
        "qcuNorm2MRHS": ([P, P, I, I], I),
        "qcuNorm2MRHSNoAlloc": ([P, P, I, S, I, P], I),
        "qcuBlasMRHS": ([I, P, P, P, P, I, P, I, P, I, S, I, P], I),
        "qcuCheckWaitTimeout": ([D], I),
        "qcuDslashSegments": ([ctypes.POINTER(QcuHopSegment), I, I, I, P], I),
        "qcuServerCreate": ([ctypes.POINTER(ctypes.c_void_p), S, I, I, I], I),
        "qcuServerAddGauge": ([P, I, ctypes.POINTER(I), I, P, I], I),
        "qcuServerSubmit": ([P, I, D, D, I, PP, PP, ctypes.POINTER(ctypes.c_longlong)], I),
        "qcuServerWait": ([P, ctypes.c_longlong, D, ctypes.POINTER(QcuRequestInfo)], I),
        "qcuServerStats": ([P, ctypes.POINTER(QcuServerStats)], I),
        "qcuServerDestroy": ([P], I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _p(x):
    return ctypes.c_void_p(int(x)) if x is not None else None


def _ptrs(xs):
    arr = (ctypes.c_void_p * len(xs))(*[int(x) for x in xs])
    return ctypes.cast(arr, ctypes.POINTER(ctypes.c_void_p)), arr


def last_error():
    L = lib()
    return L.qcuGetLastError(), (L.qcuGetLastErrorString() or b"").decode()


def clear_error():
    lib().qcuClearError()


def _raise_if(code=None):
    L = lib()
    c = L.qcuGetLastError() if code is None else code
    if c != 0:
        msg = (L.qcuGetLastErrorString() or b"").decode()
        L.qcuClearError()
        raise QcuError(c, msg)


def _param(L4):
    p = QcuParam()
    for i in range(4):
        p.lattice_size[i] = int(L4[i])
    return p


# ---- the reference's C ABI (void functions; errors raise QcuError) ----------
def initGridSize(lattice, nColors: int = 3, grid=(1, 1, 1, 1)) -> None:
    clear_error()
    g = QcuGrid()
    for i in range(4):
        g.grid_size[i] = int(grid[i])
    p = _param(lattice)
    lib().initGridSize(ctypes.byref(g), ctypes.byref(p), int(nColors))
    _raise_if()


def loadQcuGauge(gauge_ptr) -> None:
    clear_error()
    lib().loadQcuGauge(_p(gauge_ptr))
    _raise_if()


def getDslash(dslashType: int, mass: float, nColors: int, nInputs: int, floatPrecision: int) -> None:
    clear_error()
    lib().getDslash(int(dslashType), float(mass), int(nColors), int(nInputs), int(floatPrecision))
    _raise_if()


def pushBackFermions(fermionOut_ptr, fermionIn_ptr) -> None:
    clear_error()
    lib().pushBackFermions(_p(fermionOut_ptr), _p(fermionIn_ptr))
    _raise_if()


def startDslash(parity: int, daggerFlag: int = 0) -> None:
    clear_error()
    lib().startDslash(int(parity), int(daggerFlag))
    _raise_if()


def dslashQcu(out_ptr, in_ptr, gauge_ptr, lattice, parity: int) -> None:
    clear_error()
    p = _param(lattice)
    lib().dslashQcu(_p(out_ptr), _p(in_ptr), _p(gauge_ptr), ctypes.byref(p), int(parity))
    _raise_if()


def fullDslashQcu(out_ptr, in_ptr, gauge_ptr, lattice, dagger_flag: int) -> None:
    clear_error()
    p = _param(lattice)
    lib().fullDslashQcu(_p(out_ptr), _p(in_ptr), _p(gauge_ptr), ctypes.byref(p), int(dagger_flag))
    _raise_if()


def cg_inverter(x_ptr, b_ptr, gauge_ptr, lattice, p_max_prec: float, p_kappa: float) -> None:
    clear_error()
    p = _param(lattice)
    lib().cg_inverter(_p(x_ptr), _p(b_ptr), _p(gauge_ptr), ctypes.byref(p), float(p_max_prec), float(p_kappa))
    _raise_if()


# ---- extensions ----------------------------------------------------------
def set_antiperiodic_t(flag: bool) -> None:
    _raise_if(lib().qcuSetAntiperiodicT(int(bool(flag))))


def set_stream(stream_handle) -> None:
    _raise_if(lib().qcuSetStream(_p(stream_handle) if stream_handle else None))


def synchronize() -> None:
    _raise_if(lib().qcuSynchronize())


def field_bytes(precision: int, nrhs: int):
    d, n = ctypes.c_size_t(), ctypes.c_size_t()
    _raise_if(lib().qcuFieldBytes(int(precision), int(nrhs), ctypes.byref(d), ctypes.byref(n)))
    return d.value, n.value


def pack_fermions(dst, dst_norm, srcs, src_mode: int, parity: int, precision: int) -> None:
    pp, keep = _ptrs(srcs)
    _raise_if(lib().qcuPackFermions(_p(dst), _p(dst_norm), pp, len(srcs), int(src_mode), int(parity),
                                    int(precision)))


def unpack_fermions(dsts, src, src_norm, dst_mode: int, parity: int, precision: int) -> None:
    pp, keep = _ptrs(dsts)
    _raise_if(lib().qcuUnpackFermions(pp, _p(src), _p(src_norm), len(dsts), int(dst_mode), int(parity),
                                      int(precision)))


def load_gauge_lex(ptr) -> None:
    _raise_if(lib().qcuLoadGaugeLex(_p(ptr)))


def lex_to_eo(eo_out, lex_in, ncomp: int) -> None:
    _raise_if(lib().qcuLexToEo(_p(eo_out), _p(lex_in), int(ncomp)))


def eo_to_lex(lex_out, eo_in, ncomp: int) -> None:
    _raise_if(lib().qcuEoToLex(_p(lex_out), _p(eo_in), int(ncomp)))


def dslash_mrhs(out, out_norm, inp, in_norm, nrhs: int, parity: int, dagger: int, precision: int) -> None:
    _raise_if(lib().qcuDslashMRHS(_p(out), _p(out_norm), _p(inp), _p(in_norm), int(nrhs), int(parity), int(dagger),
                                  int(precision)))


def dslash_xpay_mrhs(out, out_norm, inp, in_norm, x, x_norm, nrhs: int, parity: int, dagger: int, precision: int,
                     a: float, b: float) -> None:
    _raise_if(lib().qcuDslashXpayMRHS(_p(out), _p(out_norm), _p(inp), _p(in_norm), _p(x), _p(x_norm), int(nrhs),
                                      int(parity), int(dagger), int(precision), float(a), float(b)))


def dslash_segments(segments, n_colors: int, precision: int, stream=None) -> None:
    """The hop term on several (lattice, gauge, fields) segments in one launch
    (qcuDslashSegments).  `segments`: dicts with keys lattice, gauge,
    gauge_two_row (or None), in_, out, x (or None), a, b, nrhs, parity,
    dagger, antiperiodic_t; pointers are device addresses."""
    arr = (QcuHopSegment * max(1, len(segments)))()
    for i, d in enumerate(segments):
        g = arr[i]
        g.lattice = (ctypes.c_int * 4)(*d["lattice"])
        g.gauge, g.gauge_two_row = d["gauge"], d.get("gauge_two_row")
        g.in_, g.out, g.x = d["in_"], d["out"], d.get("x")
        g.a, g.b = d.get("a", 1.0), d.get("b", 0.0)
        g.nrhs, g.parity, g.dagger = d["nrhs"], d.get("parity", 0), d.get("dagger", 0)
        g.antiperiodic_t = int(bool(d.get("antiperiodic_t", False)))
    _raise_if(lib().qcuDslashSegments(arr, len(segments), int(n_colors), int(precision), _p(stream)))


def check_wait_timeout(limit_seconds: float) -> int:
    """Run the device-side bounded-wait diagnostic (qcuCheckWaitTimeout);
    returns its status code, QCU_ERR_DEVICE_TIMEOUT (9) when the bound works."""
    return lib().qcuCheckWaitTimeout(float(limit_seconds))


def norm2_mrhs(out, field, precision: int, nrhs: int) -> None:
    """out[r] = |field_r|^2 into a device array of nrhs doubles (qcuNorm2MRHS)."""
    _raise_if(lib().qcuNorm2MRHS(_p(out), _p(field), int(precision), int(nrhs)))


BLAS_AXPBY, BLAS_AXPBYPCZ, BLAS_AXPBY_NORM, BLAS_NORM2, BLAS_NORM2_FP32, BLAS_CDOT, BLAS_ADD_TO, BLAS_COPY = range(8)


def blas_mrhs(op: int, n_elements: int, nrhs: int, x, x_precision: int, y=None, y_precision: int = 2, z=None,
              z_precision: int = 2, a=None, b=None, c=None, out=None) -> None:
    """One BLAS-1 operation on MRHS fields (qcuBlasMRHS); pointers are device
    addresses (or None), coefficients device arrays of nrhs complex doubles."""
    _raise_if(lib().qcuBlasMRHS(int(op), _p(a), _p(b), _p(c), _p(x), int(x_precision), _p(y), int(y_precision),
                                _p(z), int(z_precision), int(n_elements), int(nrhs), _p(out)))


def tune_dslash(nrhs: int, precision: int):
    """(R, block, reg_cap, packed, stages, recon, linktma) of the tuned
    kernel; stages > 0: the TMA-staged kernel, -v: tensor-core variant v (1-3
    projected half-spinor operands, 4-6 the spinor block as the MMA operand);
    recon: two-row SU(3) links; linktma: links staged by TMA per x-row."""
    R, B, M, K, T, C, X = (ctypes.c_int() for _ in range(7))
    _raise_if(lib().qcuTuneDslash(int(nrhs), int(precision), ctypes.byref(R), ctypes.byref(B), ctypes.byref(M),
                                  ctypes.byref(K), ctypes.byref(T), ctypes.byref(C), ctypes.byref(X)))
    return R.value, B.value, M.value, K.value, T.value, C.value, X.value


def last_dslash_shape():
    """(R, reg_cap, packed, stages, recon, linktma) of the kernel this
    thread's last dslash launched, after the dispatcher's fallbacks."""
    arr = (ctypes.c_int * 6)()
    _raise_if(lib().qcuLastDslashShape(arr))
    return tuple(arr)


def dslash_kernels(precision: int, n_colors: int = 3):
    """Compiled dslash kernel shapes [(R, reg_cap, packed, stages, recon,
    linktma), ...]; stages > 0: the TMA-staged kernel, -v: tensor-core variant
    v (1-6); recon: two-row SU(3) links; linktma: links staged by TMA per
    x-row."""
    arr = (ctypes.c_int * (6 * 96))()
    cnt = ctypes.c_int()
    _raise_if(lib().qcuDslashKernels(int(precision), int(n_colors), arr, 96, ctypes.byref(cnt)))
    return [tuple(arr[6 * i:6 * i + 6]) for i in range(min(cnt.value, 96))]


def load_clover(clover_ptr) -> None:
    """qcuLoadClover: clover field [2][Vh][2][2N][2N] complex double (device)."""
    _raise_if(lib().qcuLoadClover(_p(clover_ptr)))


def clover_mrhs(out, out_norm, inp, in_norm, nrhs: int, parity: int, inverse: int, precision: int) -> None:
    _raise_if(lib().qcuCloverMRHS(_p(out), _p(out_norm), _p(inp), _p(in_norm), int(nrhs), int(parity),
                                  int(inverse), int(precision)))


def measure_fma_rate(precision: int) -> float:
    """FMA throughput of the current GPU in TFLOP/s (FP64 or FP32)."""
    v = ctypes.c_double()
    _raise_if(lib().qcuMeasureFmaRate(int(precision), ctypes.byref(v)))
    return v.value


def solver_params(**kw) -> QcuSolverParam:
    p = QcuSolverParam()
    lib().qcuSolverParamDefaults(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def invert(xs, bs, params: QcuSolverParam, raise_on_error: bool = True) -> QcuSolverParam:
    px, kx = _ptrs(xs)
    pb, kb = _ptrs(bs)
    rc = lib().qcuInvert(px, pb, len(xs), ctypes.byref(params))
    if raise_on_error:
        _raise_if(rc)
    else:
        clear_error()
    return params


class Server:
    """Solve server (qcuServer*): resident gauge fields, HBM-budget admission,
    continuous MRHS batching, p50/p99 latency."""

    def __init__(self, hbm_budget_bytes: int, max_slots: int = 24, inner_precision: int = QCU_SINGLE_PRECISION,
                 solver: int = QCU_SOLVER_CG):
        h = ctypes.c_void_p()
        _raise_if(lib().qcuServerCreate(ctypes.byref(h), int(hbm_budget_bytes), int(max_slots),
                                        int(inner_precision), int(solver)))
        self.h = h
        self._keep = {}

    def add_gauge(self, gauge_id: int, lattice, n_colors: int, gauge_ptr, antiperiodic_t: bool = False) -> None:
        L = (ctypes.c_int * 4)(*[int(v) for v in lattice])
        _raise_if(lib().qcuServerAddGauge(self.h, int(gauge_id), L, int(n_colors), _p(gauge_ptr),
                                          int(bool(antiperiodic_t))))

    def submit(self, gauge_id: int, kappa: float, tol: float, xs, bs) -> int:
        px, kx = _ptrs(xs)
        pb, kb = _ptrs(bs)
        rid = ctypes.c_longlong()
        _raise_if(lib().qcuServerSubmit(self.h, int(gauge_id), float(kappa), float(tol), len(xs), px, pb,
                                        ctypes.byref(rid)))
        self._keep[rid.value] = (kx, kb)
        return rid.value

    def wait(self, request_id: int, timeout_s: float = -1.0) -> QcuRequestInfo:
        info = QcuRequestInfo()
        _raise_if(lib().qcuServerWait(self.h, ctypes.c_longlong(request_id), float(timeout_s), ctypes.byref(info)))
        if info.done:
            self._keep.pop(request_id, None)
        return info

    def stats(self) -> QcuServerStats:
        st = QcuServerStats()
        _raise_if(lib().qcuServerStats(self.h, ctypes.byref(st)))
        return st

    def close(self) -> None:
        if self.h:
            _raise_if(lib().qcuServerDestroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
