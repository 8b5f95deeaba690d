"""Helpers shared by the GPU tests: device copies and C-ABI call sequences."""
import numpy as np


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).cuda()


def abi_dslash(torch, Q, psi, gauge, L, parity, dagger=0, prec=2, antiperiodic_t=False, mass=0.0):
    """Reference call sequence of src/test.cu: initGridSize -> loadQcuGauge ->
    getDslash -> pushBackFermions (per RHS) -> startDslash."""
    nrhs, vh, _, n = psi.shape
    Q.initGridSize(L, n)
    Q.set_antiperiodic_t(antiperiodic_t)
    dg = dev(torch, gauge)
    Q.loadQcuGauge(dg.data_ptr())
    Q.getDslash(Q.DSLASH_WILSON, mass, n, nrhs, prec)
    ins = [dev(torch, psi[r]) for r in range(nrhs)]
    outs = [torch.zeros_like(x) for x in ins]
    for r in range(nrhs):
        Q.pushBackFermions(outs[r].data_ptr(), ins[r].data_ptr())
    Q.startDslash(parity, dagger)
    torch.cuda.synchronize()
    return np.stack([o.cpu().numpy() for o in outs])


TOL = {2: 1e-13, 1: 1e-6, 0: 5e-3, 4: 5e-3, 5: 5e-3}
