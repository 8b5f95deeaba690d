"""CPU check of the tensor-core dslash formulation (csrc/dslash_tc.cuh): the
real-matrix operands A, A', B, B' built the way the kernel builds them (rows
m = 2r + u; K index 2b + c = Re / Im of input colour b; N index 2a + c = Re /
Im of output colour a; zero padded to 16; A' rows swapped and signed, B'
times +-i), multiplied and accumulated over the eight hops in FP64,
reproduce the oracle's hop term."""
import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O


def gsign(mu, r):
    if mu == 0:
        return 1 if r < 2 else -1
    if mu == 1:
        return -1 if r in (0, 3) else 1
    if mu == 2:
        return 1 if r in (0, 3) else -1
    return 1


def tc_hop(psi, g, L, p, dagger, antiperiodic):
    nrhs, vh, _, N = psi.shape
    hx, Ly, Lz, Lt = L[0] // 2, L[1], L[2], L[3]
    plane, cube = hx * Ly, hx * Ly * Lz
    f = -1.0 if dagger else 1.0
    out = np.zeros_like(psi)
    for site in range(vh):
        xh, rest = site % hx, site // hx
        y, rest2 = rest % Ly, rest // Ly
        z, t = rest2 % Lz, rest2 // Lz
        eo = (y + z + t) & 1
        d_up = np.zeros((2 * nrhs, 16))
        d_lo = np.zeros((2 * nrhs, 16))
        for d in range(8):
            mu, fwd, bc = d >> 1, (d & 1) == 0, 1.0
            if mu == 0:
                if fwd:
                    nb = (site - (hx - 1) if xh == hx - 1 else site + 1) if eo != p else site
                else:
                    nb = (site + (hx - 1) if xh == 0 else site - 1) if eo == p else site
            elif mu == 1:
                nb = (site - (Ly - 1) * hx if y == Ly - 1 else site + hx) if fwd else \
                     (site + (Ly - 1) * hx if y == 0 else site - hx)
            elif mu == 2:
                nb = (site - (Lz - 1) * plane if z == Lz - 1 else site + plane) if fwd else \
                     (site + (Lz - 1) * plane if z == 0 else site - plane)
            else:
                nb = (site - (Lt - 1) * cube if t == Lt - 1 else site + cube) if fwd else \
                     (site + (Lt - 1) * cube if t == 0 else site - cube)
                if antiperiodic and (t == Lt - 1 if fwd else t == 0):
                    bc = -1.0
            w_link = g[mu, p, site] if fwd else g[mu, 1 - p, nb]
            imag, s = mu in (0, 2), (-f if fwd else f)
            a_up = np.zeros((2 * nrhs, 16))
            a_lo = np.zeros((2 * nrhs, 16))
            for r in range(nrhs):
                for u in range(2):
                    up = 3 - u if mu < 2 else u ^ 2
                    k = s * gsign(mu, u)
                    x, yv = psi[r, nb, u], psi[r, nb, up]
                    h = ((x.real - k * yv.imag) + 1j * (x.imag + k * yv.real)) if imag else x + k * yv
                    h = h * bc
                    row = np.zeros(16)
                    row[0:2 * N:2], row[1:2 * N:2] = h.real, h.imag
                    a_up[2 * r + u] = row
                    a_lo[2 * r + (up - 2)] = s * gsign(mu, up) * row
            b = np.zeros((16, 16))
            for a in range(N):
                for bb in range(N):
                    w = w_link[a, bb] if fwd else np.conj(w_link[bb, a])
                    wr, wi = w.real, w.imag
                    # re t_a += wr re h_b - wi im h_b; im t_a += wi re h_b + wr im h_b
                    b[2 * bb, 2 * a], b[2 * bb + 1, 2 * a] = wr, -wi
                    b[2 * bb, 2 * a + 1], b[2 * bb + 1, 2 * a + 1] = wi, wr
            # B' = B for real gamma rows; i t = (-im t, re t) for imaginary ones
            b2 = b.copy()
            if imag:
                b2[:, 0:2 * N:2], b2[:, 1:2 * N:2] = -b[:, 1:2 * N:2], b[:, 0:2 * N:2]
            d_up += a_up @ b
            d_lo += a_lo @ b2
        for r in range(nrhs):
            for u in range(2):
                out[r, site, u] = d_up[2 * r + u, 0:2 * N:2] + 1j * d_up[2 * r + u, 1:2 * N:2]
                out[r, site, 2 + u] = d_lo[2 * r + u, 0:2 * N:2] + 1j * d_lo[2 * r + u, 1:2 * N:2]
    return out


@pytest.mark.parametrize("n", [4, 8])
@pytest.mark.parametrize("parity,dagger,ap", [(0, 0, True), (1, 1, True), (1, 0, False)])
def test_tensor_core_operands_reproduce_the_hop(n, parity, dagger, ap):
    L = (4, 2, 2, 4)
    g = S.random_gauge(L, n, seed=11)
    psi = S.random_fermions(L, n, 3, seed=12)
    got = tc_hop(psi, g, L, parity, dagger, ap)
    ref = O.dslash(psi, g, L, parity, dagger, ap)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-13


# ---- spinor-operand formulation (csrc/dslash_tcs.cuh) -------------------------
#
# A[m][k]: m = 2 r + ri (RHS r, Re / Im part ri), k = 8 s' + b (input spin s',
# colour b padded to 8) -- the neighbour block exactly as it sits in memory.
# B[k][n]: n = 32 part + 8 s + a (part 0 / 1 = Re / Im of K_hop), the real
# split of K_hop^T, K_hop[(s, a)][(s', b)] = bc P[s][s'] W[a][b], built in
# 16-byte chunks (fixed n, 8 consecutive k = one input spin) as signed copies
# of the rows Re W[a][.] / Im W[a][.], read from the site's link record
# (link_records).  D = sum over hops of A B; the
# epilogue forms Re out = D[(r,Re)][ReK] - D[(r,Im)][ImK] and
# Im out = D[(r,Im)][ReK] + D[(r,Re)][ImK].

def chunk_code(mu, fwd, s, g, dagger, bc):
    """(source part swap, sign) of the B chunk for output spin s, input spin
    g, or None for a zero chunk -- the selection the kernel makes."""
    perm = 3 - s if mu < 2 else s ^ 2
    if g == s:
        return False, bc  # z = bc
    if g != perm:
        return None
    sg = (-1 if fwd else 1) * gsign(mu, s) * (-1 if dagger else 1) * bc
    return mu in (0, 2), sg  # z = sg * (i if imaginary gamma row)


def eo_neighbour(site, d, p, L):
    """Index of the neighbour of even-odd site `site` (parity p) for hop
    d = 2 mu + (backward), in the other parity's half-field."""
    hx, Ly, Lz, Lt = L[0] // 2, L[1], L[2], L[3]
    plane, cube = hx * Ly, hx * Ly * Lz
    xh, rest = site % hx, site // hx
    y, rest2 = rest % Ly, rest // Ly
    z, t = rest2 % Lz, rest2 // Lz
    eo = (y + z + t) & 1
    mu, fwd = d >> 1, (d & 1) == 0
    if mu == 0:
        if fwd:
            return (site - (hx - 1) if xh == hx - 1 else site + 1) if eo != p else site
        return (site + (hx - 1) if xh == 0 else site - 1) if eo == p else site
    if mu == 1:
        return (site - (Ly - 1) * hx if y == Ly - 1 else site + hx) if fwd else \
               (site + (Ly - 1) * hx if y == 0 else site - hx)
    if mu == 2:
        return (site - (Lz - 1) * plane if z == Lz - 1 else site + plane) if fwd else \
               (site + (Lz - 1) * plane if z == 0 else site - plane)
    return (site - (Lt - 1) * cube if t == Lt - 1 else site + cube) if fwd else \
           (site + (Lt - 1) * cube if t == 0 else site - cube)


def link_records(g, L):
    """The spinor-operand kernel's per-site link records (layout.h
    gauge_tc_records_bf16), in FP64: [parity][Vh][hop 8][part 2][row 8][col 8].
    Hop 2 mu holds the rows of U_mu(x) (the site's own parity), hop 2 mu + 1
    the rows of U_mu(x - mu)^T, the link of the backward neighbour (other
    parity); part 0 / 1 = Re / Im, rows and columns >= N zero."""
    N = g.shape[-1]
    vh = g.shape[2]
    rec = np.zeros((2, vh, 8, 2, 8, 8))
    for p in range(2):
        for site in range(vh):
            for d in range(8):
                mu = d >> 1
                if d & 1:
                    u = g[mu, 1 - p, eo_neighbour(site, d, p, L)].T
                else:
                    u = g[mu, p, site]
                rec[p, site, d, 0, :N, :N] = u.real
                rec[p, site, d, 1, :N, :N] = u.imag
    return rec


def tcs_hop(psi, g, L, p, dagger, antiperiodic):
    nrhs, vh, _, N = psi.shape
    hx, Ly, Lz, Lt = L[0] // 2, L[1], L[2], L[3]
    cube = hx * Ly * Lz
    records = link_records(g, L)
    out = np.zeros_like(psi)
    for site in range(vh):
        t = site // cube
        d = np.zeros((2 * nrhs, 64))
        for hop in range(8):
            mu, fwd, bc = hop >> 1, (hop & 1) == 0, 1.0
            nb = eo_neighbour(site, hop, p, L)
            if mu == 3 and antiperiodic and (t == Lt - 1 if fwd else t == 0):
                bc = -1.0
            # rows Re W[a][.], Im W[a][.] from the site's record: W = U (forward), or
            # conj(U^T) (backward), whose Im rows the builders negate
            wrow = records[p, site, hop].copy()
            if not fwd:
                wrow[1] = -wrow[1]
            a_op = np.zeros((2 * nrhs, 32))
            for r in range(nrhs):
                for sp in range(4):
                    a_op[2 * r, 8 * sp:8 * sp + N] = psi[r, nb, sp].real
                    a_op[2 * r + 1, 8 * sp:8 * sp + N] = psi[r, nb, sp].imag
            b_op = np.zeros((32, 64))
            for c in range(256):  # the kernel's chunk numbering
                a, gs, s, part = c & 7, (c >> 3) & 3, (c >> 5) & 3, c >> 7
                code = chunk_code(mu, fwd, s, gs, dagger, bc)
                if code is None:
                    continue
                imag, sg = code
                src = part ^ int(imag)
                # z = sg (real): part -> sg * row part; z = sg * i: Re -> -sg Im W, Im -> +sg Re W
                neg = (sg < 0) if not imag else ((sg > 0) if part == 0 else (sg < 0))
                b_op[8 * gs:8 * gs + 8, 32 * part + 8 * s + a] = (-1 if neg else 1) * wrow[src, a]
            d += a_op @ b_op
        for r in range(nrhs):
            re = d[2 * r, 0:32] - d[2 * r + 1, 32:64]
            im = d[2 * r + 1, 0:32] + d[2 * r, 32:64]
            for sp in range(4):
                out[r, site, sp] = re[8 * sp:8 * sp + N] + 1j * im[8 * sp:8 * sp + N]
    return out


@pytest.mark.parametrize("n", [3, 4, 8])
@pytest.mark.parametrize("parity,dagger,ap", [(0, 0, True), (1, 1, True), (1, 0, False), (0, 1, False)])
def test_spinor_operand_formulation_reproduces_the_hop(n, parity, dagger, ap):
    L = (4, 2, 2, 4)
    g = S.random_gauge(L, n, seed=13)
    psi = S.random_fermions(L, n, 3, seed=14)
    got = tcs_hop(psi, g, L, parity, dagger, ap)
    ref = O.dslash(psi, g, L, parity, dagger, ap)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-13


@pytest.mark.parametrize("L", [(4, 2, 2, 4), (6, 4, 2, 2), (2, 2, 2, 2)])
def test_link_records_hold_every_link_twice(L):
    """The per-site records hold each link twice: as rows of U in its own
    site's forward hop, and transposed in exactly one backward hop of the
    other parity (the site it is the backward neighbour of)."""
    n = 3
    g = S.random_gauge(L, n, seed=21)
    rec = link_records(g, L)
    vh = g.shape[2]
    for p in range(2):
        for mu in range(4):
            fwd = rec[p, :, 2 * mu, 0, :n, :n] + 1j * rec[p, :, 2 * mu, 1, :n, :n]
            assert np.array_equal(fwd, g[mu, p])
            bwd = rec[p, :, 2 * mu + 1, 0, :n, :n] + 1j * rec[p, :, 2 * mu + 1, 1, :n, :n]
            nbs = [eo_neighbour(s, 2 * mu + 1, p, L) for s in range(vh)]
            assert sorted(nbs) == list(range(vh))  # a permutation of the other parity's sites
            for s in range(vh):
                assert np.array_equal(bwd[s], g[mu, 1 - p, nbs[s]].T)
