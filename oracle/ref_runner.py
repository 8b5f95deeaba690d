"""Run the reference's own device code (rebuilt by ``oracle/build_ref.sh``)
through the CUDA driver API.

TEST INFRASTRUCTURE ONLY: used to pin the oracle against the reference
(``tests/golden/make_golden.py``) and by GPU tests that compare against the
reference kernel when ``oracle/_ref/`` is present.  Device memory comes from
torch; kernels are launched with ``cuLaunchKernel`` on torch's current stream.

Reference internal ("coalesced") layouts the kernels expect
(include/basic_data/qcu_point.cuh:80-88, include/kernels/storageLoadStore/
loadAndStore.cuh:6-15,41-62):
  fermion per RHS  [4N][Vh] complex
  gauge            [4][2][N*N][Vh] complex
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")

# kernels instantiated in oracle/ref_shim.cu: (precision tag, N) -> nrhs values
DSLASH_VARIANTS = {("d", 3): (1, 2, 3, 4, 5), ("f", 3): (1, 4), ("d", 4): (2,), ("f", 4): (2,),
                   ("d", 5): (1,), ("f", 5): (1,)}


def available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "qcuref.cubin")) or \
        os.path.exists(os.path.join(REF_DIR, "qcuref.ptx"))


def expected() -> bool:
    """True when build_ref.sh found the reference sources: the module must
    then exist, and a missing module is a build failure, not a skip."""
    return os.path.exists(os.path.join(REF_DIR, "expected"))


def require(pytest) -> None:
    """Skip when the reference was never available to build; fail when it
    was and the module is missing."""
    if available():
        return
    if expected():
        pytest.fail("the reference sources were present but oracle/_ref/ holds no module "
                    "(oracle/build_ref.sh failed)")
    pytest.skip("reference module not built (oracle/build_ref.sh found no reference sources)")


class RefModule:
    def __init__(self):
        import torch
        torch.zeros(1, device="cuda")  # make torch's primary context current
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + \
            [ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.module = ctypes.c_void_p()
        errs = []
        self.loaded_from = None
        for fname in ("qcuref.cubin", "qcuref.ptx"):
            path = os.path.join(REF_DIR, fname)
            if not os.path.exists(path):
                continue
            data = open(path, "rb").read()
            if fname.endswith(".ptx"):
                data += b"\0"
            rc = self.cu.cuModuleLoadData(ctypes.byref(self.module), data)
            if rc == 0:
                self.loaded_from = fname
                break
            errs.append("%s: CUresult %d" % (fname, rc))
        if self.loaded_from is None:
            raise RuntimeError("cannot load the reference module: " + "; ".join(errs or ["not built"]))
        names_file = os.path.join(REF_DIR, "names.txt")
        self.names = open(names_file).read().split() if os.path.exists(names_file) else []

    def function(self, name: str):
        f = ctypes.c_void_p()
        rc = self.cu.cuModuleGetFunction(ctypes.byref(f), self.module, name.encode())
        if rc != 0:
            raise RuntimeError("cuModuleGetFunction(%s) -> %d" % (name, rc))
        return f

    def launch(self, name: str, grid: int, block: int, args) -> None:
        f = self.function(name)
        holders = list(args)
        ptrs = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p)
                                                  for h in holders])
        stream = self.torch.cuda.current_stream().cuda_stream
        rc = self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, ctypes.c_void_p(stream), ptrs, None)
        if rc != 0:
            raise RuntimeError("cuLaunchKernel(%s) -> %d" % (name, rc))

    def _storage(self, which: str) -> str:
        for n in self.names:
            if which in n:
                return n
        raise RuntimeError("storage kernel %s not in names.txt" % which)

    # --- the reference's storage (layout) kernels, double SU(3) only --------
    def store_vector_coalesced(self, psi: np.ndarray, L) -> np.ndarray:
        """storeVectorCoalesced<double,3> (storage_kernels.cuh:14-32) on one RHS
        (Vh, 4, 3) -> (12, Vh)."""
        torch = self.torch
        vh = psi.shape[0]
        src = torch.from_numpy(np.ascontiguousarray(psi, np.complex128)).cuda()
        dst = torch.empty((12, vh), dtype=torch.complex128, device="cuda")
        self.launch(self._storage("storeVectorCoalesced"), (vh + 255) // 256, 256,
                    [ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                     ctypes.c_int(L[0] // 2), ctypes.c_int(L[1]), ctypes.c_int(L[2]), ctypes.c_int(L[3])])
        torch.cuda.synchronize()
        return dst.cpu().numpy()

    def store_vector_noncoalesced(self, soa: np.ndarray, L) -> np.ndarray:
        torch = self.torch
        vh = soa.shape[1]
        src = torch.from_numpy(np.ascontiguousarray(soa, np.complex128)).cuda()
        dst = torch.empty((vh, 4, 3), dtype=torch.complex128, device="cuda")
        self.launch(self._storage("storeVectorNonCoalesced"), (vh + 255) // 256, 256,
                    [ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                     ctypes.c_int(L[0] // 2), ctypes.c_int(L[1]), ctypes.c_int(L[2]), ctypes.c_int(L[3])])
        torch.cuda.synchronize()
        return dst.cpu().numpy()

    def store_gauge_coalesced(self, gauge: np.ndarray, L) -> np.ndarray:
        """storeGaugeCoalesced<double,3> (storage_kernels.cuh:54-76):
        (4, 2, Vh, 3, 3) -> (4, 2, 9, Vh)."""
        torch = self.torch
        vh = gauge.shape[2]
        src = torch.from_numpy(np.ascontiguousarray(gauge, np.complex128)).cuda()
        dst = torch.empty((4, 2, 9, vh), dtype=torch.complex128, device="cuda")
        self.launch(self._storage("storeGaugeCoalesced"), (vh + 255) // 256, 256,
                    [ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                     ctypes.c_int(L[0]), ctypes.c_int(L[1]), ctypes.c_int(L[2]), ctypes.c_int(L[3])])
        torch.cuda.synchronize()
        return dst.cpu().numpy()

    def store_gauge_noncoalesced(self, soa: np.ndarray, L) -> np.ndarray:
        torch = self.torch
        vh = soa.shape[-1]
        src = torch.from_numpy(np.ascontiguousarray(soa, np.complex128)).cuda()
        dst = torch.empty((4, 2, vh, 3, 3), dtype=torch.complex128, device="cuda")
        self.launch(self._storage("storeGaugeNonCoalesced"), (vh + 255) // 256, 256,
                    [ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                     ctypes.c_int(L[0]), ctypes.c_int(L[1]), ctypes.c_int(L[2]), ctypes.c_int(L[3])])
        torch.cuda.synchronize()
        return dst.cpu().numpy()

    # --- the reference's dslash ---------------------------------------------
    def dslash(self, psi: np.ndarray, gauge: np.ndarray, L, parity: int, dagger: int = 0, prec: str = "d",
               antiperiodic_t: bool = False) -> np.ndarray:
        """Reference applyWilson on (nrhs, Vh, 4, N) caller-layout spinors.

        Antiperiodic time boundaries are obtained the only way the reference
        allows: U_t negated on the t = Lt-1 slice before the call."""
        torch = self.torch
        nrhs, vh, _, n = psi.shape
        if nrhs not in DSLASH_VARIANTS.get((prec, n), ()):
            raise ValueError("no reference instantiation for prec=%s N=%d nrhs=%d" % (prec, n, nrhs))
        g = np.array(gauge, dtype=np.complex128, copy=True)
        if antiperiodic_t:
            Lx, Ly, Lz, Lt = L
            tsl = (np.arange(vh) // (Lx // 2 * Ly * Lz)) == Lt - 1
            g[3, :, tsl] *= -1.0
        cdt = np.complex128 if prec == "d" else np.complex64
        tdt = torch.complex128 if prec == "d" else torch.complex64
        g_soa = np.ascontiguousarray(g.reshape(4, 2, vh, n * n).transpose(0, 1, 3, 2)).astype(cdt)
        dg = torch.from_numpy(g_soa).cuda()
        ins, outs = [], []
        for r in range(nrhs):
            soa = np.ascontiguousarray(psi[r].reshape(vh, 4 * n).T).astype(cdt)
            ins.append(torch.from_numpy(soa).cuda())
            outs.append(torch.zeros((4 * n, vh), dtype=tdt, device="cuda"))

        class Mrhs(ctypes.Structure):
            _fields_ = [("fermion", ctypes.c_void_p * nrhs)]

        o = Mrhs()
        i = Mrhs()
        for r in range(nrhs):
            o.fermion[r] = outs[r].data_ptr()
            i.fermion[r] = ins[r].data_ptr()
        flag = (ctypes.c_double if prec == "d" else ctypes.c_float)(-1.0 if dagger else 1.0)
        self.launch("qcuref_dslash_%s_%d_%d" % (prec, n, nrhs), (vh + 255) // 256, 256,
                    [o, i, ctypes.c_void_p(dg.data_ptr()), flag, ctypes.c_int(L[0]), ctypes.c_int(L[1]),
                     ctypes.c_int(L[2]), ctypes.c_int(L[3]), ctypes.c_int(parity)])
        torch.cuda.synchronize()
        res = np.stack([outs[r].cpu().numpy().T.reshape(vh, 4, n) for r in range(nrhs)])
        return res.astype(np.complex128)
