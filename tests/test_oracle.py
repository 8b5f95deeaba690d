"""CPU tests of the FP64 oracle: pinned against the reference's own GPU
kernel outputs (tests/golden/, made by tests/golden/make_golden.py), against
an independent dense-gamma restatement, and against the identities the
operator must satisfy."""
import json
import os

import numpy as np
import pytest

from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as fh:
        return json.load(fh)


def test_golden_manifest_pinned():
    m = manifest()
    assert m["all_ok"]
    assert all(m["storage"].values()), "reference storage kernels must equal plain transposes"
    for case in m["cases"]:
        for c in case["combos"]:
            tol = case.get("tol", 1e-13)
            assert c["oracle_vs_ref_rel_l2"] < tol


def test_golden_full_fixture():
    """Oracle vs the reference kernel's stored outputs, bit-for-bit inputs."""
    m = manifest()
    case = [c for c in m["cases"] if c["name"] == "su3_d_4x4x4x8_full"][0]
    data = np.load(os.path.join(GOLDEN, case["file"]))
    g, psi, L = data["gauge"], data["psi"], tuple(case["L"])
    for c in case["combos"]:
        out = O.dslash(psi, g, L, c["parity"], c["dagger"], c["antiperiodic_t"])
        assert rel(out, data[c["key"]]) < 1e-13


@pytest.mark.parametrize("name", ["config0_su3_d_8x8x8x8_nrhs4_apt", "su3_d_8x8x8x8_nrhs5_periodic",
                                  "su3_f_8x8x8x8_nrhs4", "su4_d_4x4x4x8_nrhs2", "su4_f_4x4x4x8_nrhs2",
                                  "su5_d_4x4x4x8_nrhs1", "su5_f_4x4x4x8_nrhs1", "su3_d_6x4x4x4_nrhs3_oddtail"])
def test_golden_checksums(name):
    """Oracle vs the reference kernel through seeded inputs + stored checksums."""
    from tests.golden.make_golden import projections  # noqa: WPS433
    m = manifest()
    case = [c for c in m["cases"] if c["name"] == name][0]
    chk = np.load(os.path.join(GOLDEN, m["checksums_file"]))
    L, n, nrhs = tuple(case["L"]), case["N"], case["nrhs"]
    g = S.random_gauge(L, n, seed=case["gauge_seed"])
    psi = S.random_fermions(L, n, nrhs, seed=case["psi_seed"])
    tol = max(case["tol"], 1e-12)
    for c in case["combos"]:
        out = O.dslash(psi, g, L, c["parity"], c["dagger"], c["antiperiodic_t"])
        ref_norm = chk[c["key"] + "_norm"]
        np.testing.assert_allclose([np.linalg.norm(out[k]) for k in range(nrhs)], ref_norm, rtol=tol)
        head = chk[c["key"] + "_head"]
        assert rel(out[:, :head.shape[1]], head) < 10 * tol
        proj = projections(out, c["proj_seed"])
        scale = np.linalg.norm(out) * np.sqrt(out[0].size)
        assert np.max(np.abs(proj - chk[c["key"] + "_proj"])) < 10 * tol * scale


@pytest.mark.parametrize("n", [3, 4, 5, 8])
@pytest.mark.parametrize("ap", [False, True])
def test_oracle_matches_dense_gamma(n, ap):
    L = (4, 2, 2, 4)
    g = S.random_gauge(L, n, seed=3)
    psi = S.random_fermions(L, n, 2, seed=4)
    for parity in (0, 1):
        for dag in (0, 1):
            a = O.dslash(psi, g, L, parity, dag, ap)
            b = O.dslash_dense_gamma(psi, g, L, parity, dag, ap)
            assert rel(a, b) < 1e-14


def test_gamma_algebra():
    gam = O.gammas()
    for m in range(4):
        assert np.allclose(gam[m], gam[m].conj().T)
        for n in range(4):
            ac = gam[m] @ gam[n] + gam[n] @ gam[m]
            assert np.allclose(ac, 2 * np.eye(4) * (m == n))
    g5 = gam[0] @ gam[1] @ gam[2] @ gam[3]
    assert np.allclose(g5, np.diag([1, 1, -1, -1]))


def test_free_field_plane_wave():
    """U = 1: a plane wave e^{ipx} u is an eigenvector of the hop with
    eigen-matrix sum_mu 2 (cos p_mu - i f sin p_mu gamma_mu)."""
    L = (4, 4, 4, 8)
    n = 2
    Lx, Ly, Lz, Lt = L
    g = S.unit_gauge(L, n)
    k = np.array([1, 2, 3, 1])
    p = 2 * np.pi * k / np.array(L)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((4, n)) + 1j * rng.standard_normal((4, n))
    vh = S.half_volume(L)
    gam = O.gammas()
    for parity in (0, 1):
        for dag in (0, 1):
            f = -1 if dag else 1
            idx = np.arange(vh)
            xh = idx % (Lx // 2)
            y = (idx // (Lx // 2)) % Ly
            z = (idx // (Lx // 2 * Ly)) % Lz
            t = idx // (Lx // 2 * Ly * Lz)
            def phase(par):
                X = 2 * xh + (par ^ ((y + z + t) & 1))
                return np.exp(1j * (p[0] * X + p[1] * y + p[2] * z + p[3] * t))

            psi_in = (phase(1 - parity)[:, None, None] * u[None])[None]
            out = O.dslash(psi_in, g, L, parity, dag)[0]
            mat = sum(2 * (np.cos(p[m]) * np.eye(4) - 1j * f * np.sin(p[m]) * gam[m]) for m in range(4))
            expect = phase(parity)[:, None, None] * np.einsum("st,ta->sa", mat, u)[None]
            assert rel(out, expect) < 1e-13


def test_gamma5_hermiticity():
    """<y, D_eo x> = <gamma5 D_oe^f gamma5 ... > : D^dag (f=+1) equals the f=-1 hop."""
    L = (4, 4, 2, 4)
    n = 3
    g = S.random_gauge(L, n, seed=5)
    x = S.random_fermions(L, n, 1, seed=6)
    y = S.random_fermions(L, n, 1, seed=7)
    # <y_even, D_eo x_odd> == <D_oe^{f=-1} y_even, x_odd>
    lhs = np.vdot(y, O.dslash(x, g, L, 0, 0))
    rhs = np.vdot(O.dslash(y, g, L, 1, 1), x)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


def test_gauge_covariance():
    """D(U^Omega) Omega psi = Omega D(U) psi for a random local SU(N) rotation."""
    L = (4, 2, 4, 2)
    n = 3
    vh = S.half_volume(L)
    g = S.random_gauge(L, n, seed=8)
    psi = S.random_fermions(L, n, 1, seed=9)
    rng = np.random.default_rng(10)
    om = S.random_sun(2 * vh, n, rng).reshape(2, vh, n, n)  # Omega[parity][site]
    Lx, Ly, Lz, Lt = L

    def nb(parity, i, mu):
        xh = i % (Lx // 2)
        y = (i // (Lx // 2)) % Ly
        z = (i // (Lx // 2 * Ly)) % Lz
        t = i // (Lx // 2 * Ly * Lz)
        c = [2 * xh + (parity ^ ((y + z + t) & 1)), y, z, t]
        c[mu] = (c[mu] + 1) % L[mu]
        return ((c[3] * Lz + c[2]) * Ly + c[1]) * (Lx // 2) + c[0] // 2

    g2 = np.empty_like(g)
    for mu in range(4):
        for par in range(2):
            for i in range(vh):
                j = nb(par, i, mu)
                g2[mu, par, i] = om[par, i] @ g[mu, par, i] @ om[1 - par, j].conj().T
    for parity in (0, 1):
        rot_in = np.einsum("vab,rvsb->rvsa", om[1 - parity], psi)
        lhs = O.dslash(rot_in, g2, L, parity, 0)
        rhs = np.einsum("vab,rvsb->rvsa", om[parity], O.dslash(psi, g, L, parity, 0))
        assert rel(lhs, rhs) < 1e-13


def test_mrhs_linearity():
    """The nrhs-batched oracle equals per-RHS applications bitwise."""
    L = (4, 4, 4, 4)
    g = S.random_gauge(L, 3, seed=11)
    psi = S.random_fermions(L, 3, 3, seed=12)
    batch = O.dslash(psi, g, L, 1, 0, True)
    for r in range(3):
        one = O.dslash(psi[r:r + 1], g, L, 1, 0, True)
        assert np.array_equal(batch[r], one[0])


def test_lex_eo_roundtrip():
    L = (4, 2, 6, 2)
    rng = np.random.default_rng(13)
    V = 4 * 2 * 6 * 2
    lex = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    eo = O.lex_to_eo(lex, L)
    assert eo.shape == (2, V // 2, 4, 3)
    assert np.array_equal(O.eo_to_lex(eo, L), lex)
    # parity of lexicographic site (X, y, z, t) -> ((X+y+z+t) & 1)
    X, y, z, t = 3, 1, 4, 1
    s = ((t * 6 + z) * 2 + y) * 4 + X
    i = ((t * 6 + z) * 2 + y) * 2 + X // 2
    assert np.array_equal(eo[(X + y + z + t) & 1, i], lex[s])


def test_oracle_cgnr_solves_wilson():
    L = (4, 4, 2, 2)
    n = 3
    g = S.random_gauge(L, n, seed=14)
    b = S.random_fermions(L, n, 1, seed=15, parities=2)[0]
    x, it, res = O.cgnr_full(b, g, L, 0.12, tol=1e-11, maxiter=2000)
    assert res < 1e-11
    assert O.true_residual(x, b, g, L, 0.12) == pytest.approx(res, rel=1e-6)
