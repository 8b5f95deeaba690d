"""Generate the golden fixtures that pin the FP64 oracle to the reference.

Runs on a machine with a GPU and a built ``oracle/_ref/`` (see
``oracle/build_ref.sh``): every case below is computed by the reference's own
device code (``oracle/ref_runner.py``) and by the oracle, the two are
compared, and the reference's outputs are written as fixtures:

* full outputs for a small 4x4x4x8 SU(3) lattice (inputs stored too);
* for larger or other-N cases, seeds plus checksums (checksums.npz): K
  seeded random complex projections of each output RHS, its L2 norm, and its
  first sites in full.

Usage:  python tests/golden/make_golden.py OUTDIR
The committed copies live in tests/golden/ beside this script.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mrhs_qcu_gb300 import synthetic as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import ref_runner  # noqa: E402

K_PROJ = 8
HEAD_SITES = 16


def projections(out: np.ndarray, seed: int) -> np.ndarray:
    """(nrhs, K) complex projections of each RHS onto seeded random vectors."""
    nrhs = out.shape[0]
    flat = out.reshape(nrhs, -1)
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((K_PROJ, flat.shape[1])) + 1j * rng.standard_normal((K_PROJ, flat.shape[1]))
    return flat @ w.T


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def main(outdir: str) -> int:
    os.makedirs(outdir, exist_ok=True)
    ref = ref_runner.RefModule()
    manifest = {"loaded_from": ref.loaded_from, "cases": [], "storage": {}}
    ok = True

    # 1. storage kernels (layout transforms), bitwise against plain transposes
    L = (4, 4, 4, 8)
    g = S.random_gauge(L, 3, seed=11)
    psi = S.random_fermions(L, 3, 1, seed=12)[0]
    soa = ref.store_vector_coalesced(psi, L)
    back = ref.store_vector_noncoalesced(soa, L)
    gsoa = ref.store_gauge_coalesced(g, L)
    gback = ref.store_gauge_noncoalesced(gsoa, L)
    vh = psi.shape[0]
    st = {
        "vector_to_coalesced_exact": bool(np.array_equal(soa, psi.reshape(vh, 12).T)),
        "vector_roundtrip_exact": bool(np.array_equal(back, psi)),
        "gauge_to_coalesced_exact": bool(np.array_equal(gsoa, g.reshape(4, 2, vh, 9).transpose(0, 1, 3, 2))),
        "gauge_roundtrip_exact": bool(np.array_equal(gback, g)),
    }
    manifest["storage"] = st
    ok &= all(st.values())
    print("storage:", st)

    # 2. full fixture: small SU(3) FP64 lattice, nrhs=2
    L = (4, 4, 4, 8)
    g = S.random_gauge(L, 3, seed=21)
    psi = S.random_fermions(L, 3, 2, seed=22)
    arrays = {"gauge": g, "psi": psi}
    combos = [(0, 0, False), (1, 0, False), (0, 1, False), (1, 1, False), (0, 0, True), (1, 1, True)]
    case = {"name": "su3_d_4x4x4x8_full", "L": L, "N": 3, "nrhs": 2, "prec": "d", "file": "su3_d_4x4x4x8.npz",
            "combos": []}
    for parity, dagger, ap in combos:
        r = ref.dslash(psi, g, L, parity, dagger, "d", ap)
        o = O.dslash(psi, g, L, parity, dagger, ap)
        e = rel(o, r)
        key = "out_p%d_d%d_ap%d" % (parity, dagger, int(ap))
        arrays[key] = r
        case["combos"].append({"parity": parity, "dagger": dagger, "antiperiodic_t": ap, "key": key,
                               "oracle_vs_ref_rel_l2": e})
        ok &= e < 1e-13
        print(case["name"], parity, dagger, ap, e)
    np.savez_compressed(os.path.join(outdir, case["file"]), **arrays)
    manifest["cases"].append(case)

    # 3. checksum fixtures: (name, L, N, nrhs, prec, gauge seed, psi seed, combos, tol)
    specs = [
        ("config0_su3_d_8x8x8x8_nrhs4_apt", (8, 8, 8, 8), 3, 4, "d", 31, 32,
         [(0, 0, True), (1, 0, True), (0, 1, True), (1, 1, True)], 1e-13),
        ("su3_d_8x8x8x8_nrhs5_periodic", (8, 8, 8, 8), 3, 5, "d", 41, 42, [(1, 0, False), (0, 1, False)], 1e-13),
        ("su3_f_8x8x8x8_nrhs4", (8, 8, 8, 8), 3, 4, "f", 51, 52, [(0, 0, False), (1, 1, True)], 1e-6),
        ("su4_d_4x4x4x8_nrhs2", (4, 4, 4, 8), 4, 2, "d", 61, 62, [(0, 0, False), (1, 1, True)], 1e-13),
        ("su4_f_4x4x4x8_nrhs2", (4, 4, 4, 8), 4, 2, "f", 63, 64, [(1, 0, False)], 1e-6),
        ("su5_d_4x4x4x8_nrhs1", (4, 4, 4, 8), 5, 1, "d", 71, 72, [(0, 1, False), (1, 0, True)], 1e-13),
        ("su5_f_4x4x4x8_nrhs1", (4, 4, 4, 8), 5, 1, "f", 73, 74, [(0, 0, False)], 1e-6),
        ("su3_d_6x4x4x4_nrhs3_oddtail", (6, 4, 4, 4), 3, 3, "d", 81, 82, [(0, 0, False), (1, 1, True)], 1e-13),
    ]
    checks = {}
    for name, L, n, nrhs, prec, gs, ps, combos, tol in specs:
        g = S.random_gauge(L, n, seed=gs)
        psi = S.random_fermions(L, n, nrhs, seed=ps)
        case = {"name": name, "L": L, "N": n, "nrhs": nrhs, "prec": prec, "gauge_seed": gs, "psi_seed": ps,
                "tol": tol, "combos": []}
        for i, (parity, dagger, ap) in enumerate(combos):
            r = ref.dslash(psi, g, L, parity, dagger, prec, ap)
            o = O.dslash(psi, g, L, parity, dagger, ap)
            e = rel(o, r)
            pseed = 1000 + i
            key = "%s_c%d" % (name, i)
            checks[key + "_proj"] = projections(r, pseed)
            checks[key + "_norm"] = np.array([np.linalg.norm(r[k]) for k in range(nrhs)])
            checks[key + "_head"] = r[:, :HEAD_SITES]
            case["combos"].append({
                "parity": parity, "dagger": dagger, "antiperiodic_t": ap, "oracle_vs_ref_rel_l2": e,
                "proj_seed": pseed, "key": key,
            })
            ok &= e < tol
            print(name, parity, dagger, ap, e)
        manifest["cases"].append(case)

    np.savez_compressed(os.path.join(outdir, "checksums.npz"), **checks)
    manifest["checksums_file"] = "checksums.npz"
    manifest["all_ok"] = bool(ok)
    with open(os.path.join(outdir, "manifest.json"), "w") as fh:
        json.dump(manifest, fh, indent=1)
    print("all_ok", ok)
    return 0 if ok else 1


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py OUTDIR")
    sys.exit(main(sys.argv[1]))
