"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle reproduces the committed fixtures exactly (regression pin).
GPU: the library's matrices match them bit for bit and its FP64 iterates
within 1e-10 relative.
"""
import ast
import glob
import os

import numpy as np
import pytest

from conftest import rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def load(path):
    z = np.load(path)
    meta = ast.literal_eval(str(z["meta"]))  # dict literal written by make_golden
    return z, meta


def oracle_build(O, meta, theta):
    if meta["kind"] == "parallel":
        return O.paralleltomo(meta["n"], meta["nth"], meta["p"], theta)
    return O.fanlineartomo(meta["n"], meta["nth"], meta["p"], meta["r"], meta["dw"], meta["sd"],
                           theta, geometry_fix=meta["fix"])


def gpu_build(F, meta, theta):
    d = F.Data(n=meta["n"], p=meta["p"], nth=meta["nth"], r=meta.get("r", 0.0),
               dw=meta.get("dw", 0.0), sd=meta.get("sd", 0.0), theta=theta)
    if meta["kind"] == "parallel":
        return F.paralleltomo(d)
    return F.fanlineartomo(d, geometry_fix=meta["fix"])


def test_fixtures_present():
    assert len(FILES) >= 5


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_oracle_reproduces_golden(oracle, path):
    z, meta = load(path)
    R = oracle_build(oracle, meta, z["theta"])
    assert np.array_equal(R.IA, z["IA"]) and np.array_equal(R.JA, z["JA"])
    assert np.array_equal(R.vA, z["vA"])
    T = oracle.reorder(R)
    assert np.array_equal(T.IA, z["TIA"]) and np.array_equal(T.JA, z["TJA"])
    b = z["b"]
    x = oracle.sirt("cimmino", R, b, 10, opts=oracle.options(relaxpar=1.5, lbound=0.0))
    assert np.array_equal(x, z["sirt_cimmino"])
    X = oracle.art("kaczmarz", R, b, [2], opts=oracle.options(relaxpar=0.25))
    assert np.array_equal(X[:, 0], z["kaczmarz"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_gpu_matches_golden(fair, path):
    z, meta = load(path)
    A = gpu_build(fair, meta, z["theta"])
    vA, IA, JA = A.arrays()
    assert np.array_equal(IA, z["IA"]) and np.array_equal(JA, z["JA"])
    assert np.max(np.abs(vA - z["vA"]) / np.maximum(np.abs(z["vA"]), 1e-300), initial=0) <= 1e-12
    b = z["b"]
    o = fair.airms.options
    assert rel_err(fair.airms.sirt("cimmino", A, b, 10, opts=o(relaxpar=1.5, lbound=0.0)),
                   z["sirt_cimmino"]) < 1e-10
    assert rel_err(fair.airms.sirt("sart", A, b, 10, opts=o(lbound=0.0, ubound=1.0)),
                   z["sirt_sart"]) < 1e-10
    assert rel_err(fair.airms.art("kaczmarz", A, b, [2], opts=o(relaxpar=0.25))[:, 0],
                   z["kaczmarz"]) < 1e-10
    assert rel_err(fair.airms.art("symkaczmarz", A, b, [2], opts=o(relaxpar=0.5, lbound=0.0))[:, 0],
                   z["symkaczmarz"]) < 1e-10
    A.transpose()
    tv, tIA, tJA = A.arrays()
    assert np.array_equal(tIA, z["TIA"]) and np.array_equal(tJA, z["TJA"])
    assert np.array_equal(tv, z["TvA"])
