"""Seeded synthetic lattice fields in the caller layouts of ``qcu.h``.

* Links: Haar-random SU(N) -- QR of an N x N complex-Gaussian matrix with the
  phases of R's diagonal moved into Q (so Q is Haar-distributed on U(N)), then
  divided by det(Q)^(1/N) so that det = 1.
* Spinors: i.i.d. complex Gaussian, unit variance per spin-colour component
  (real and imaginary parts each of variance 1/2).
* Point sources: a unit entry at one (site, spin, colour) per RHS.

Layouts (complex128):
  gauge   (4, 2, Vh, N, N)   [mu][parity][half-site][row][col]
  fermion (nrhs, Vh, 4, N)   one parity per RHS
  full    (nrhs, 2, Vh, 4, N) even half first
These are the caller ("non-coalesced") layouts of the reference
(include/kernels/storage/storage_kernels.cuh:14-101).
"""
from __future__ import annotations

import numpy as np


def half_volume(L) -> int:
    Lx, Ly, Lz, Lt = [int(v) for v in L]
    if Lx % 2:
        raise ValueError("Lx must be even for an even-odd split")
    return Lx * Ly * Lz * Lt // 2


def random_sun(count: int, n: int, rng: np.random.Generator, chunk: int = 1 << 20) -> np.ndarray:
    """``count`` Haar-random SU(n) matrices, shape (count, n, n), complex128.

    Modified Gram-Schmidt on the columns equals the QR factorisation with a
    positive real R diagonal, i.e. the phase-fixed QR."""
    out = np.empty((count, n, n), dtype=np.complex128)
    for s in range(0, count, chunk):
        e = min(count, s + chunk)
        m = e - s
        a = (rng.standard_normal((m, n, n)) + 1j * rng.standard_normal((m, n, n))) * np.sqrt(0.5)
        q = np.empty_like(a)
        for k in range(n):
            v = a[:, :, k].copy()
            for j in range(k):
                proj = np.einsum("mi,mi->m", np.conj(q[:, :, j]), v)
                v -= proj[:, None] * q[:, :, j]
            v /= np.linalg.norm(v, axis=1)[:, None]
            q[:, :, k] = v
        det = np.linalg.det(q)
        q *= (det ** (-1.0 / n))[:, None, None]
        out[s:e] = q
    return out


def random_gauge(L, n: int = 3, seed: int = 0) -> np.ndarray:
    vh = half_volume(L)
    rng = np.random.default_rng(seed)
    return random_sun(4 * 2 * vh, n, rng).reshape(4, 2, vh, n, n)


def unit_gauge(L, n: int = 3) -> np.ndarray:
    vh = half_volume(L)
    g = np.zeros((4, 2, vh, n, n), dtype=np.complex128)
    g[..., np.arange(n), np.arange(n)] = 1.0
    return g


def random_fermions(L, n: int, nrhs: int, seed: int = 1, parities: int = 1) -> np.ndarray:
    """Gaussian spinors: (nrhs, Vh, 4, n) for one parity, or
    (nrhs, 2, Vh, 4, n) when ``parities == 2``."""
    vh = half_volume(L)
    rng = np.random.default_rng(seed)
    shape = (nrhs, vh, 4, n) if parities == 1 else (nrhs, 2, vh, 4, n)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * np.sqrt(0.5)


def point_sources(L, n: int, nrhs: int, seed: int = 2) -> np.ndarray:
    """Unit point sources at seeded random (site, spin, colour), full lattice
    in eo layout: (nrhs, 2, Vh, 4, n)."""
    vh = half_volume(L)
    rng = np.random.default_rng(seed)
    b = np.zeros((nrhs, 2, vh, 4, n), dtype=np.complex128)
    for r in range(nrhs):
        p = int(rng.integers(2))
        site = int(rng.integers(vh))
        spin = int(rng.integers(4))
        col = int(rng.integers(n))
        b[r, p, site, spin, col] = 1.0
    return b


def random_sun_torch(count: int, n: int, generator, device="cuda", chunk: int = 1 << 20):
    """Haar-random SU(n) on a torch device with elementwise ops only (no
    linear-algebra library): modified Gram-Schmidt of complex-Gaussian
    columns (the phase-fixed QR), then division by det^(1/n), the
    determinant from Gaussian elimination with partial pivoting."""
    import torch
    out = torch.empty((count, n, n), dtype=torch.complex128, device=device)
    for s in range(0, count, chunk):
        m = min(chunk, count - s)
        re = torch.randn((m, n, n), generator=generator, device=device, dtype=torch.float64)
        im = torch.randn((m, n, n), generator=generator, device=device, dtype=torch.float64)
        q = torch.complex(re, im) * (0.5 ** 0.5)
        for k in range(n):
            v = q[:, :, k].clone()
            for j in range(k):
                qj = q[:, :, j]
                v = v - (qj.conj() * v).sum(-1, keepdim=True) * qj
            q[:, :, k] = v / v.abs().pow(2).sum(-1, keepdim=True).sqrt()
        a = q.clone()
        det = torch.ones(m, dtype=torch.complex128, device=device)
        rows = torch.arange(m, device=device)
        for k in range(n):
            piv = a[:, k:, k].abs().argmax(dim=1) + k
            swap = piv != k
            rk = a[rows, k].clone()
            rp = a[rows, piv].clone()
            a[rows, k] = rp
            a[rows, piv] = rk
            det = torch.where(swap, -det, det) * a[:, k, k]
            if k + 1 < n:
                f = a[:, k + 1:, k] / a[:, k, k].unsqueeze(1)
                a[:, k + 1:, :] -= f.unsqueeze(2) * a[:, k:k + 1, :]
        out[s:s + m] = q * (det ** (-1.0 / n)).view(-1, 1, 1)
    return out


def random_clover(L, n: int, eps: float = 0.1, seed: int = 3) -> np.ndarray:
    """A clover-like field: per site two Hermitian (2n x 2n) blocks
    1 + eps * H, H Hermitian with Gaussian entries, in the caller layout
    (2, Vh, 2, 2n, 2n) complex double (positive definite for small eps)."""
    vh = half_volume(L)
    rng = np.random.default_rng(seed)
    m = 2 * n
    h = rng.standard_normal((2, vh, 2, m, m)) + 1j * rng.standard_normal((2, vh, 2, m, m))
    h = 0.5 * (h + np.conj(np.swapaxes(h, -1, -2)))
    return np.eye(m, dtype=np.complex128) + eps * h
