"""The main.exe drop-in (fortran_airtools_gb300/_lib/fair_main) on the GPU.

Test mode (main.f90:190-220: N=256, 400 angles over linspace(0, pi), 384
bins, Shepp-Logan, 0.5% noise) is rerun with the oracle from the same
stream seed, and sol.txt / errorgauge.txt must match the oracle's results
(the files carry 17 significant digits); the matrix file written by -s is
the oracle's matrix bit for bit and -r reproduces the run; -I runs the
input-file mode of main.f90:222-271 on a small fan-beam data file.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fortran_airtools_gb300", "_lib", "fair_main")


def run(args, cwd, seed):
    env = dict(os.environ, FAIR_SEED=str(seed))
    r = subprocess.run([EXE] + args, cwd=cwd, capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stderr
    return r


@pytest.fixture(scope="module")
def test_problem(oracle):
    """The oracle's test-mode problem, with the first stream seed whose noise
    draws the Newton inverse converges on (it fails on some upper-tail draws
    with this libm: the reference stops there too)."""
    th = oracle.linspace(0.0, np.pi, 400)
    R = oracle.paralleltomo_mt(256, 400, 384, th, os.cpu_count() or 1)
    x = oracle.shepplogan(256)
    b = oracle.matvecmul(R, x)
    for seed in range(8):
        oracle.random_seed(seed)
        try:
            bt, _ = oracle.add_white_noise(b, 5e-3)
        except Exception:
            continue
        return R, x, bt, seed
    pytest.skip("no seed with a converging noise draw")


def test_sirt_matches_oracle(test_problem, oracle, tmp_path):
    R, x, bt, seed = test_problem
    run(["-t", "-K5", "-Mcimmino", "-osol.txt"], tmp_path, seed)
    sol = np.loadtxt(tmp_path / "sol.txt")
    assert sol.size == R.n
    assert rel_err(sol, oracle.sirt("cimmino", R, bt, 5)) < 1e-10


def test_kaczmarz_default_method(test_problem, oracle, tmp_path):
    R, x, bt, seed = test_problem
    run(["-t", "-K2"], tmp_path, seed)
    sol = np.loadtxt(tmp_path / "sol.txt")
    assert rel_err(sol, oracle.art("kaczmarz", R, bt, [2])[:, 0]) < 1e-10


def test_errorgauge_output(test_problem, oracle, tmp_path):
    R, x, bt, seed = test_problem
    run(["-t", "-K6", "-Seg", "-R0.5"], tmp_path, seed)
    eg = np.loadtxt(tmp_path / "errorgauge.txt")
    sol = np.loadtxt(tmp_path / "sol.txt")
    o = oracle.options(relaxpar=0.5)
    xo, fi, _, _, EG = oracle.twin_art("kaczmarz", "errorgauge", R, bt, [6], opts=o)
    assert eg.size == 6
    assert rel_err(eg, EG) < 1e-8
    assert rel_err(sol, xo) < 1e-10


def test_store_and_read_matrix(test_problem, fair, tmp_path):
    import ctypes as C
    R, x, bt, seed = test_problem
    run(["-t", "-K3", "-Mcimmino", "-smat.bin", "-osol_s.txt"], tmp_path, seed)
    L = fair.lib()
    m, n, nz = C.c_int32(), C.c_int32(), C.c_int32()
    f = str(tmp_path / "mat.bin").encode()
    assert L.fair_read_csr_file_sizes(f, C.byref(m), C.byref(n), C.byref(nz)) == 0
    assert (m.value, n.value, nz.value) == (R.m, R.n, R.nnz)
    vA, JA, IA = np.empty(R.nnz), np.empty(R.nnz, np.int32), np.empty(R.m + 1, np.int32)
    assert L.fair_read_csr_file(f, vA.ctypes.data, JA.ctypes.data, IA.ctypes.data) == 0
    assert np.array_equal(IA, R.IA) and np.array_equal(JA, R.JA) and np.array_equal(vA, R.vA)
    run(["-t", "-K3", "-Mcimmino", "-rmat.bin", "-osol_r.txt"], tmp_path, seed)
    assert open(tmp_path / "sol_s.txt").read() == open(tmp_path / "sol_r.txt").read()


def test_input_file_mode(oracle, tmp_path):
    """-I: read_data, grid scaling, fanlineartomo, A scaled by grid_size/N,
    b = -log(T) (main.f90:222-271), then SART."""
    n, nth, p, r, dw, sd = 32, 36, 46, 2.0, 3.0, 4.0
    deg = 10.0 * np.arange(nth)
    gs = dw * r / sd
    R = oracle.fanlineartomo(n, nth, p, r / gs, dw / gs, sd / gs, deg / 180.0 * np.pi)
    R.vA = R.vA * (gs / n)
    T = np.exp(-oracle.matvecmul(R, oracle.shepplogan(n)))
    lines = [f"n {n}", f"p {p}", f"nth {nth}", f"R {r!r}", f"dw {dw!r}", f"sd {sd!r}", f"theta {nth}"]
    lines += [repr(float(v)) for v in deg] + [f"T {T.size}"] + [repr(float(v)) for v in T]
    (tmp_path / "in.txt").write_text("\n".join(lines) + "\n")
    run(["-Iin.txt", "-Msart", "-K10", "-L0"], tmp_path, 0)
    sol = np.loadtxt(tmp_path / "sol.txt")
    xr = oracle.sirt("sart", R, -np.log(T), 10, opts=oracle.options(lbound=0.0))
    assert rel_err(sol, xr) < 1e-10


def test_random_phantom_test_mode(test_problem, oracle, tmp_path):
    """-tgrains: the phantom's seeds are drawn before the noise, from the
    same stream, as choose_phantom precedes add_white_noise (main.f90:213-215)."""
    R, _, _, seed = test_problem
    for s in range(seed, seed + 8):
        oracle.random_seed(s)
        x = oracle.phantom("grains", 256)
        try:
            bt, _ = oracle.add_white_noise(oracle.matvecmul(R, x), 5e-3)
        except Exception:
            continue
        run(["-tgrains", "-K4", "-Mcimmino"], tmp_path, s)
        sol = np.loadtxt(tmp_path / "sol.txt")
        assert rel_err(sol, oracle.sirt("cimmino", R, bt, 4)) < 1e-10
        return
    pytest.skip("no seed with a converging noise draw")
