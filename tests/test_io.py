"""File formats of the reference's driver (include/fair_io.h) and the
main.exe drop-in's argument handling, on the CPU.

Matrix files are checked byte for byte against the gfortran unformatted
sequential layout of store_matrix (system_generation.f90:595-627): six
records framed by 4-byte length markers; the reader also takes a record
split into gfortran subrecords (negative markers). Text files follow
list-directed READ rules (main.f90 / read_data).
"""
import ctypes as C
import os
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "fortran_airtools_gb300", "_lib", "fair_main")


@pytest.fixture(scope="module")
def L(fair):
    return fair.lib()


def rec(b):
    return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))


def small_csr():
    IA = np.array([0, 2, 2, 5], np.int32)
    JA = np.array([1, 3, 2, 3, 4], np.int32)
    vA = np.array([0.5, 1.25, -2.0, 3.0, 1e-3])
    return 3, 4, vA, JA, IA


def test_matrix_file_layout_and_round_trip(L, tmp_path):
    m, n, vA, JA, IA = small_csr()
    f = str(tmp_path / "A.bin").encode()
    assert L.fair_write_csr_file(f, m, n, 5, vA.ctypes.data, JA.ctypes.data, IA.ctypes.data) == 0
    want = (rec(struct.pack("<i", m)) + rec(struct.pack("<i", n)) + rec(struct.pack("<i", 5))
            + rec(vA.tobytes()) + rec(JA.tobytes()) + rec(IA.tobytes()))
    assert open(f, "rb").read() == want
    mm, nn, nz = C.c_int32(), C.c_int32(), C.c_int32()
    assert L.fair_read_csr_file_sizes(f, C.byref(mm), C.byref(nn), C.byref(nz)) == 0
    assert (mm.value, nn.value, nz.value) == (m, n, 5)
    v2, J2, I2 = np.empty(5), np.empty(5, np.int32), np.empty(m + 1, np.int32)
    assert L.fair_read_csr_file(f, v2.ctypes.data, J2.ctypes.data, I2.ctypes.data) == 0
    assert np.array_equal(v2, vA) and np.array_equal(J2, JA) and np.array_equal(I2, IA)


def test_matrix_file_subrecords(L, tmp_path):
    """A vA record split in two gfortran subrecords: the first with a negative
    leading marker, the second with a negative trailing marker."""
    m, n, vA, JA, IA = small_csr()
    b = vA.tobytes()
    a1, a2 = b[:16], b[16:]
    split = (struct.pack("<i", -len(a1)) + a1 + struct.pack("<i", len(a1))
             + struct.pack("<i", len(a2)) + a2 + struct.pack("<i", -len(a2)))
    data = (rec(struct.pack("<i", m)) + rec(struct.pack("<i", n)) + rec(struct.pack("<i", 5))
            + split + rec(JA.tobytes()) + rec(IA.tobytes()))
    f = tmp_path / "S.bin"
    f.write_bytes(data)
    v2, J2, I2 = np.empty(5), np.empty(5, np.int32), np.empty(m + 1, np.int32)
    assert L.fair_read_csr_file(str(f).encode(), v2.ctypes.data, J2.ctypes.data, I2.ctypes.data) == 0
    assert np.array_equal(v2, vA)
    bad = tmp_path / "B.bin"  # markers that disagree
    bad.write_bytes(data[:-4] + struct.pack("<i", 99))
    assert L.fair_read_csr_file(str(bad).encode(), v2.ctypes.data, J2.ctypes.data, I2.ctypes.data) == 4


def test_read_data_list_directed(fair, L, tmp_path):
    """read_data (system_generation.f90:494-539): name/value lines, a value
    may sit on the next line, extra items on a line are dropped, D exponents."""
    text = ("n 4 extra\np 3\nnth\n2\nR 2.5d0\ndw 1.5D0, 7\nsd 1.25\n"
            "theta 2\n0.0\n90.0\n"
            "T 6\n1.0\n0.5d0\n0.25\n1e-1\n0.75\n0.125\n")
    f = tmp_path / "in.txt"
    f.write_text(text)
    n, p, nth = C.c_int32(), C.c_int32(), C.c_int32()
    assert L.fair_read_data_sizes(str(f).encode(), C.byref(n), C.byref(p), C.byref(nth)) == 0
    assert (n.value, p.value, nth.value) == (4, 3, 2)
    dat = fair.Data(n=0, p=0, nth=0)._c()
    th, T = np.empty(2), np.empty(6)
    assert L.fair_read_data(str(f).encode(), C.addressof(dat), th.ctypes.data, T.ctypes.data) == 0
    assert (dat.r, dat.dw, dat.sd) == (2.5, 1.5, 1.25)
    assert np.array_equal(th, np.array([0.0, 90.0]) / 180.0 * 3.141592653589793)
    assert np.array_equal(T, [1.0, 0.5, 0.25, 0.1, 0.75, 0.125])
    f.write_text(text.replace("theta 2", "theta 3"))
    assert L.fair_read_data(str(f).encode(), C.addressof(dat), th.ctypes.data, T.ctypes.data) == 4
    assert b"Angle vector has the wrong length" in L.fair_last_error_detail()


def test_ordering_ref_and_values(L, tmp_path):
    f = tmp_path / "ord.txt"
    f.write_text("len 4\n3\n1\n4\n2\n")
    ln = C.c_int32()
    assert L.fair_read_ordering(str(f).encode(), C.byref(ln), None, 0) == 0 and ln.value == 4
    o = np.empty(4, np.int32)
    assert L.fair_read_ordering(str(f).encode(), C.byref(ln), o.ctypes.data, 4) == 0
    assert list(o) == [3, 1, 4, 2]
    x = np.array([0.5, -1.2345678901234567e-5, 0.1, 123.456, 0.0, 2.0 ** 60, np.pi])
    g = str(tmp_path / "sol.txt")
    assert L.fair_write_values(g.encode(), x.ctypes.data, x.size) == 0
    assert np.array_equal(np.loadtxt(g), x)  # 17 significant digits round-trip
    lines = open(g).read().splitlines()
    assert lines[0] == "  0.50000000000000000     " and lines[2] == "  0.10000000000000001     "
    assert lines[1] == "  -1.2345678901234568E-005"
    r = np.empty(x.size)
    assert L.fair_read_ref(g.encode(), x.size, r.ctypes.data) == 0 and np.array_equal(r, x)


def run(args, cwd):
    return subprocess.run([EXE] + args, cwd=cwd, capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("args,msg", [
    ([], "STOP Supply input file or activate test mode."),
    (list("abcdefghij"), "STOP Too many input arguments."),
    (["-Mlandweber"], "STOP Not a recognised stopping rule. Use -h for help."),
    (["-Sfoo"], "STOP Not a recognised stopping rule. Choose from 'errorgauge' or 'mutualstep'."),
    (["-tfoo"], "STOP Not a recognised phantom in -t. Use -h for help."),
    (["-x"], "STOP Not a recognised flag, use -h for help."),
    (["-sa.bin", "-rb.bin"], "STOP Choose either storing or reading matrix."),
    (["-n-1"], "STOP Provide positive noise level."),
])
def test_cli_stops(fair, tmp_path, args, msg):
    r = run(args, tmp_path)
    assert r.returncode == 0 and r.stderr.strip() == msg


def test_cli_help_and_hamster(fair, tmp_path):
    r = run(["-h"], tmp_path)
    assert r.returncode == 0 and "Main CT AIR tools input flags:" in r.stdout
    assert "'kaczmarz', 'randkaczmarz', 'rand', 'symkaczmarz', 'sym', 'graddescent', 'gd', 'cimmino', and 'sart'." in r.stdout
    r = run(["-H"], tmp_path)
    assert r.returncode == 0 and "Oh noes, the hamster! RUN!!!" in r.stdout


def test_cli_without_gpu(fair, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = run(["-t", "-K2"], tmp_path)
    assert r.returncode == 1 and "No CUDA device" in r.stderr
