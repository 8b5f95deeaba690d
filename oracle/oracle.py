"""ctypes wrapper of the FP64 CPU oracle (``oracle/qcu_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``, to check results.  The product library
(``mrhs_qcu_gb300``) never imports it.

Array conventions (all complex128, C-contiguous), restating the reference's
caller layouts (include/kernels/storage/storage_kernels.cuh:14-101):

* gauge  ``(4, 2, Vh, N, N)``   -- [mu][parity][site][row][col]
* fermion ``(nrhs, Vh, 4, N)``  -- per RHS, one parity, [site][spin][colour]
* full-lattice eo field ``(2, Vh, 4, N)`` -- even half first
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc + OpenMP into ``oracle/_build/liboracle.so``."""
    src = os.path.join(_HERE, "qcu_oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        os.makedirs(_BUILD, exist_ok=True)
        tmp = _SO + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                               src, "-o", tmp, "-lm"])
        os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        I = ctypes.c_int
        D = ctypes.c_double
        _lib.oracle_dslash.argtypes = [P, P, P, P, I, I, I, I, I]
        _lib.oracle_lex_to_eo.argtypes = [P, P, P, I]
        _lib.oracle_eo_to_lex.argtypes = [P, P, P, I]
        _lib.oracle_clover_apply.argtypes = [P, P, P, P, I, I, I, I]
        _lib.oracle_wilson_full.argtypes = [P, P, P, P, P, I, D, I, I, P]
        _lib.oracle_cgnr_full.argtypes = [P, P, P, P, P, I, D, I, D, I, ctypes.POINTER(D)]
        _lib.oracle_cgnr_full.restype = I
        _lib.oracle_true_residual.argtypes = [P, P, P, P, P, I, D, I]
        _lib.oracle_true_residual.restype = D
        _lib.oracle_num_threads.restype = I
        _lib.oracle_set_num_threads.argtypes = [I]
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _dims(L):
    return (ctypes.c_int * 4)(*[int(v) for v in L])


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def num_threads() -> int:
    return lib().oracle_num_threads()


def set_num_threads(n: int) -> None:
    lib().oracle_set_num_threads(int(n))


def dslash(psi: np.ndarray, gauge: np.ndarray, L, parity: int, dagger: int = 0,
           antiperiodic_t: bool = False) -> np.ndarray:
    """Hopping term D_parity^f on every RHS of ``psi`` (nrhs, Vh, 4, N)."""
    psi = _c128(psi)
    gauge = _c128(gauge)
    nrhs, vh, ns, n = psi.shape
    assert ns == 4 and gauge.shape == (4, 2, vh, n, n)
    out = np.empty_like(psi)
    lib().oracle_dslash(_ptr(out), _ptr(psi), _ptr(gauge), _dims(L), n, nrhs, int(parity), int(dagger),
                        int(bool(antiperiodic_t)))
    return out


def lex_to_eo(lex: np.ndarray, L) -> np.ndarray:
    """(V, ...) lexicographic -> (2, Vh, ...) even-odd."""
    lex = _c128(lex)
    v = lex.shape[0]
    ncomp = int(np.prod(lex.shape[1:]))
    eo = np.empty((2, v // 2) + lex.shape[1:], dtype=np.complex128)
    lib().oracle_lex_to_eo(_ptr(eo), _ptr(lex), _dims(L), ncomp)
    return eo


def eo_to_lex(eo: np.ndarray, L) -> np.ndarray:
    eo = _c128(eo)
    ncomp = int(np.prod(eo.shape[2:]))
    lex = np.empty((eo.shape[0] * eo.shape[1],) + eo.shape[2:], dtype=np.complex128)
    lib().oracle_eo_to_lex(_ptr(lex), _ptr(eo), _dims(L), ncomp)
    return lex


def _clover_ptr(clover):
    """(pointer, array kept alive by the caller) of an optional clover field."""
    if clover is None:
        return None, None
    c = _c128(clover)
    return _ptr(c), c


def clover_apply(psi: np.ndarray, clover: np.ndarray, L, parity: int, dagger: int = 0) -> np.ndarray:
    """A_parity psi for psi (nrhs, Vh, 4, N); clover (2, Vh, 2, 2N, 2N)."""
    psi = _c128(psi)
    clover = _c128(clover)
    out = np.empty_like(psi)
    lib().oracle_clover_apply(_ptr(out), _ptr(psi), _ptr(clover), _dims(L), psi.shape[-1], psi.shape[0],
                              int(parity), int(dagger))
    return out


def wilson_full(x: np.ndarray, gauge: np.ndarray, L, kappa: float, dagger: int = 0,
                antiperiodic_t: bool = False, clover=None) -> np.ndarray:
    """M x = A x - kappa D x on a full eo field (2, Vh, 4, N); A = 1 without
    a clover field (2, Vh, 2, 2N, 2N)."""
    x = _c128(x)
    gauge = _c128(gauge)
    cp, keep = _clover_ptr(clover)
    n = x.shape[-1]
    out = np.empty_like(x)
    sc = np.empty(x.shape, dtype=np.complex128)
    lib().oracle_wilson_full(_ptr(out), _ptr(x), _ptr(gauge), cp, _dims(L), n, float(kappa), int(dagger),
                             int(bool(antiperiodic_t)), _ptr(sc))
    return out


def cgnr_full(b: np.ndarray, gauge: np.ndarray, L, kappa: float, tol: float = 1e-12, maxiter: int = 5000,
              antiperiodic_t: bool = False, clover=None):
    """Solve M x = b (full lattice, no preconditioning) by CGNR in FP64."""
    b = _c128(b)
    gauge = _c128(gauge)
    cp, keep = _clover_ptr(clover)
    x = np.empty_like(b)
    res = ctypes.c_double()
    it = lib().oracle_cgnr_full(_ptr(x), _ptr(b), _ptr(gauge), cp, _dims(L), b.shape[-1], float(kappa),
                                int(bool(antiperiodic_t)), float(tol), int(maxiter), ctypes.byref(res))
    return x, it, res.value


def true_residual(x: np.ndarray, b: np.ndarray, gauge: np.ndarray, L, kappa: float,
                  antiperiodic_t: bool = False, clover=None) -> float:
    """|b - M x| / |b| in FP64 for a full eo field (2, Vh, 4, N)."""
    x = _c128(x)
    b = _c128(b)
    gauge = _c128(gauge)
    cp, keep = _clover_ptr(clover)
    return lib().oracle_true_residual(_ptr(x), _ptr(b), _ptr(gauge), cp, _dims(L), b.shape[-1], float(kappa),
                                      int(bool(antiperiodic_t)))


def dslash_dense_gamma(psi: np.ndarray, gauge: np.ndarray, L, parity: int, dagger: int = 0,
                       antiperiodic_t: bool = False) -> np.ndarray:
    """Second, independent restatement in numpy with explicit 4x4 gamma
    matrices (no spin projection), for small lattices only.  Gamma matrices as
    read off include/kernels/wilson_dslash_4d.cuh:74-81,134-141,193-200,253-260."""
    psi = _c128(psi)
    nrhs, vh, _, n = psi.shape
    Lx, Ly, Lz, Lt = [int(v) for v in L]
    gam = gammas()
    one = np.eye(4)
    f = -1.0 if dagger else 1.0
    idx = np.arange(vh)
    xh = idx % (Lx // 2)
    y = (idx // (Lx // 2)) % Ly
    z = (idx // (Lx // 2 * Ly)) % Lz
    t = idx // (Lx // 2 * Ly * Lz)
    X = 2 * xh + (parity ^ ((y + z + t) & 1))
    coords = [X, y, z, t]
    out = np.zeros_like(psi)
    for mu in range(4):
        for step in (+1, -1):
            nc = [c.copy() for c in coords]
            nc[mu] = (coords[mu] + step) % L[mu]
            j = ((nc[3] * Lz + nc[2]) * Ly + nc[1]) * (Lx // 2) + nc[0] // 2
            bc = np.ones(vh)
            if antiperiodic_t and mu == 3:
                cross = (coords[3] == Lt - 1) if step == 1 else (coords[3] == 0)
                bc = np.where(cross, -1.0, 1.0)
            if step == 1:
                U = gauge[mu, parity][idx]
                proj = one - f * gam[mu]
            else:
                U = np.conj(np.swapaxes(gauge[mu, 1 - parity][j], -1, -2))
                proj = one + f * gam[mu]
            nb = psi[:, j]                                   # (nrhs, Vh, 4, N)
            col = np.einsum("vab,rvsb->rvsa", U, nb)        # colour multiply
            out += bc[None, :, None, None] * np.einsum("st,rvta->rvsa", proj, col)
    return out


def gammas() -> np.ndarray:
    """DeGrand-Rossi gamma_x, gamma_y, gamma_z, gamma_t of the reference."""
    i = 1j
    gx = np.array([[0, 0, 0, i], [0, 0, i, 0], [0, -i, 0, 0], [-i, 0, 0, 0]])
    gy = np.array([[0, 0, 0, -1], [0, 0, 1, 0], [0, 1, 0, 0], [-1, 0, 0, 0]], dtype=complex)
    gz = np.array([[0, 0, i, 0], [0, 0, 0, -i], [-i, 0, 0, 0], [0, i, 0, 0]])
    gt = np.array([[0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0], [0, 1, 0, 0]], dtype=complex)
    return np.stack([gx, gy, gz, gt])
