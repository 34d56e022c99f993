"""The C-ABI library (CPU checks, no GPU needed).

libfair_gb300.so must load and export every function declared in
include/*.h; its host-only functions (linspace, scramble, the random stream,
Shepp-Logan, add_white_noise, options) must agree bit for bit with the
oracle; without a GPU, handle creation must fail with FAIR_ERR_NOGPU.
"""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(fair_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(fair):
    L = fair.lib()
    names = declared_symbols()
    assert len(names) >= 39
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_every_symbol_has_a_signature(fair):
    """Every entry point is declared with argtypes in the bindings: an
    undeclared one would take pointer arguments as 32-bit ints."""
    import fortran_airtools_gb300._clib as clib
    src = open(clib.__file__).read()
    missing = [n for n in declared_symbols() if f'"{n}"' not in src]
    assert not missing, missing


def test_error_strings(fair):
    L = fair.lib()
    assert L.fair_error_string(1) == b"Vector input size incorrect."
    assert L.fair_error_string(3) == b"++ Something went wrong"
    assert L.fair_error_string(5) == b"Newton method did not converge."


def test_options_defaults(fair, oracle):
    """initialise_options (AIRMs.f90:29-36), including lbound=1, ubound=0."""
    o = fair.Opts().initialise()
    r = oracle.options()
    for f in ("relaxpar", "ubound", "lbound", "damp", "upb", "lwrb", "rowprobability"):
        assert getattr(o, f) == getattr(r, f)
    o.set_ubound(2.0).set_lbound(-1.0)
    assert (o.upb, o.ubound, o.lwrb, o.lbound) == (1, 2.0, 1, -1.0)


def test_host_functions_match_oracle(fair, oracle):
    from fortran_airtools_gb300 import airms, phantomgallery, system_generation
    assert np.array_equal(system_generation.linspace(0, np.pi, 400), oracle.linspace(0, np.pi, 400))
    assert np.array_equal(system_generation.linspace(-3, 5, 7), oracle.linspace(-3, 5, 7))
    for seed in (0, 7, 2 ** 40 + 3):
        airms.random_seed(seed)
        oracle.random_seed(seed)
        assert np.array_equal(airms.random_number(17), oracle.random_number(17))
        assert np.array_equal(airms.scramble(1000), oracle.scramble(1000))
    for N in (2, 5, 64, 128):
        assert np.array_equal(phantomgallery.shepplogan(N), oracle.shepplogan(N))
    b = np.linspace(0.0, 3.0, 2000)
    airms.random_seed(3)
    oracle.random_seed(3)
    g = system_generation.add_white_noise(b, 0.01)
    r = oracle.add_white_noise(b, 0.01)
    assert np.array_equal(g[0], r[0]) and np.array_equal(g[1], r[1])


def test_vectorise_is_column_major(fair):
    from fortran_airtools_gb300 import phantomgallery
    img = np.arange(6.0).reshape(2, 3)
    assert list(phantomgallery.vectorise(img)) == [0, 3, 1, 4, 2, 5]


def test_no_gpu_is_an_error(fair):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(fair.FairError) as ei:
        fair.CSRMatrix()
    assert ei.value.status == 10
    with pytest.raises(fair.FairError) as ei:
        fair.Batch("f32")
    assert ei.value.status == 10


def test_missing_library_raises(monkeypatch):
    import fortran_airtools_gb300._clib as clib
    monkeypatch.setattr(clib, "_lib_handle", None)
    monkeypatch.setattr(clib, "LIB_PATH", os.path.join(ROOT, "no_such_lib.so"))
    with pytest.raises(RuntimeError):
        clib.lib()
