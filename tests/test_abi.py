"""CPU tests of the C-ABI boundary: libqcu.so loads without a GPU, exports
every function the public headers declare, and reports host-side errors
through qcuGetLastError() instead of terminating the process (the reference
calls exit(1), include/qcu_macro.cuh:16-40)."""
import ctypes
import os
import re

import pytest

import mrhs_qcu_gb300 as Q

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", txt, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    return Q.lib()


def test_headers_declare_reference_abi():
    names = declared_functions("qcu.h")
    for n in ["initGridSize", "pushBackFermions", "startDslash", "loadQcuGauge", "getDslash", "dslashQcu",
              "fullDslashQcu", "cg_inverter"]:
        assert n in names


@pytest.mark.parametrize("header", ["qcu.h", "qcu_gb300.h"])
def test_every_declared_symbol_exported(lib, header):
    names = declared_functions(header)
    assert names
    for n in names:
        assert hasattr(lib, n), "%s declared in %s but not exported" % (n, header)
    assert set(Q.ABI_SYMBOLS + Q.EXT_SYMBOLS) >= set(declared_functions("qcu.h") + declared_functions("qcu_gb300.h"))


def test_cxx_storage_symbols_match_reference_mangling(lib):
    for sym in Q.CXX_SYMBOLS:
        assert hasattr(lib, sym)


def test_enum_values_match_reference():
    # include/qcu_enum.h:4-12 of the reference
    assert (Q.QCU_HALF_PRECISION, Q.QCU_SINGLE_PRECISION, Q.QCU_DOUBLE_PRECISION) == (0, 1, 2)
    assert (Q.EVEN_PARITY, Q.ODD_PARITY) == (0, 1)
    assert (Q.DSLASH_WILSON, Q.DSLASH_CLOVER) == (0, 1)
    assert ctypes.sizeof(Q.QcuParam) == 16 and ctypes.sizeof(Q.QcuGrid) == 16


def test_version(lib):
    assert b"sm_103a" in lib.qcuVersion()


def test_errors_are_reported_not_fatal(lib):
    """Host-side failures set an error code and return (no GPU needed)."""
    Q.clear_error()
    lib.pushBackFermions(None, None)
    code, msg = Q.last_error()
    assert code in (1, 2)
    Q.clear_error()
    with pytest.raises(Q.QcuError) as e:
        Q.initGridSize((8, 8, 8, 8), 3, grid=(2, 1, 1, 1))
    assert e.value.code == 3  # multi-process grids unsupported, not silently wrong
    with pytest.raises(Q.QcuError) as e:
        Q.initGridSize((7, 8, 8, 8), 3)
    assert e.value.code == 2
    with pytest.raises(Q.QcuError) as e:
        Q.initGridSize((8, 8, 8, 8), 9)
    assert e.value.code == 3
    Q.initGridSize((8, 8, 8, 8), 3)  # pure host work
    with pytest.raises(Q.QcuError) as e:
        Q.getDslash(0, -3.5, 3, 1, 2)
    assert e.value.code == 5  # gauge not loaded (reference: "localGauge_ is nullptr")
    with pytest.raises(Q.QcuError) as e:
        Q.startDslash(0, 0)
    assert e.value.code == 6  # no operator
    with pytest.raises(Q.QcuError):
        Q.dslash_mrhs(0, 0, 0, 0, 1, 0, 0, 7)  # bad precision


def test_solver_param_defaults(lib):
    p = Q.solver_params()
    assert p.solver == Q.QCU_SOLVER_CG and p.tol == 1e-10 and p.inner_precision == 1 and p.use_graph == 1


# ---- the reference's C++ operator interface (qcu_dirac.h, qcd/qcu_dslash.h) ----
# mangled names of the reference's declarations (include/qcu_dirac.h:40-50,
# include/qcd/qcu_dslash.h:62-64 of the reference), which a C++ caller built
# against the reference's headers links to
REFERENCE_CXX_SYMBOLS = [
    "_ZN3qcu17instantiateDslashERK11QcuLattDescILi4EERK11QcuProcDescILi4EEiidPvS8_S8_11DSLASH_TYPE"
    "13QCU_PRECISIONiiRNS_16ExecutionStreamsE",
    "_ZN3qcu11DiracWilson6DslashEPvS1_iii",
    "_ZTVN3qcu11DiracWilsonE",
    "_ZN3qcu12WilsonDslashIfLi3ELi4EE5applyEv",
    "_ZN3qcu12WilsonDslashIdLi5ELi1EE5applyEv",
]


def test_reference_operator_symbols_exported(lib):
    for sym in REFERENCE_CXX_SYMBOLS:
        assert hasattr(lib, sym), sym


def _exported_symbols():
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--defined-only", Q.lib()._name], capture_output=True, text=True).stdout
    return [line.split()[-1] for line in out.splitlines() if line.strip()]


def test_internal_symbols_hidden():
    """Only the public headers' functions and classes leave libqcu.so: no
    internal qcu:: symbol (session, solver engine, kernel launchers) is
    exported, so they cannot clash with a caller's symbols."""
    syms = _exported_symbols()
    internal = [s for s in syms if s.startswith("_ZN3qcu") and not (
        s.startswith("_ZN3qcu17instantiateDslash") or s.startswith("_ZN3qcu11DiracWilson") or
        s.startswith("_ZN3qcu12WilsonDslash") or s.startswith("_ZN3qcu6Dslash") or
        s.startswith("_ZN3qcu7storage"))]
    assert not internal, internal[:10]
    assert any(s == "initGridSize" for s in syms)


def test_cxx_caller_builds_against_public_headers(tmp_path):
    """A C++ program written against include/ (qcu_dirac.h, qcd/qcu_dslash.h,
    qcu_gb300.h) compiles with g++ and links against libqcu.so."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if gxx is None or not os.path.exists(os.path.join(cuda, "include", "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are not available")
    exe = build_cxx_caller(str(tmp_path), gxx, cuda)
    assert os.path.exists(exe)


def build_cxx_caller(outdir, gxx, cuda):
    import subprocess
    libdir = os.path.dirname(Q.lib()._name)
    exe = os.path.join(outdir, "dirac_caller")
    cmd = [gxx, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cxx", "dirac_caller.cpp"), "-o", exe, os.path.join(libdir, "libqcu.so"),
           "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe
