"""The autotuner's file cache (QCU_TUNE_CACHE) across processes: a first
process tunes and writes its choice for (precision, N, nrhs, volume); a
second process, started with a different choice planted in the file, uses
the planted shape without tuning, and its dslash still matches the oracle.
Each process is a fresh interpreter, so only the file carries the choice."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np, torch
import mrhs_qcu_gb300 as Q
from mrhs_qcu_gb300 import synthetic as S
from oracle import oracle as O
from tests.util import abi_dslash, rel
L, n, nrhs = (4, 4, 4, 8), 3, 12
g = S.random_gauge(L, n, seed=800)
psi = S.random_fermions(L, n, nrhs, seed=801)
got = abi_dslash(torch, Q, psi, g, L, 0, 0, 1, antiperiodic_t=True)
err = rel(got, O.dslash(psi, g, L, 0, 0, True))
print(json.dumps({"shape": list(Q.tune_dslash(nrhs, 1)), "err": err}))
"""


def run_child(cache):
    env = dict(os.environ, QCU_TUNE_CACHE=str(cache))
    env.pop("QCU_DSLASH_CONFIG", None)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_tune_cache_round_trip(cuda, tmp_path):
    cache = tmp_path / "tune.txt"
    first = run_child(cache)
    assert first["err"] < 1e-6
    lines = [line.split() for line in cache.read_text().splitlines() if line.strip()]
    key = "1:3:12:256"  # FP32, SU(3), 12 RHS, Vh = 4*4*4*8/2
    mine = [f for f in lines if f[0] == key]
    assert len(mine) == 1
    R, block, minb, pk = (int(v) for v in mine[0][1:5])
    assert [R, block, minb, pk] == first["shape"][:4]
    # plant another valid shape (scalar kernel, R = 1, block 64, full links) and start afresh
    planted = "%s 1 64 1 0 0 0 0 0\n" % key
    cache.write_text("".join(" ".join(f) + "\n" for f in lines if f[0] != key) + planted)
    second = run_child(cache)
    assert second["shape"][:4] == [1, 64, 1, 0] and second["shape"][5] == 0
    assert second["err"] < 1e-6
