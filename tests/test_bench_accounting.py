"""bench.py's byte accounting and kernel naming (no GPU): the algorithmic
bytes of a SIRT pass follow the layout the pass reads (CSR, packed groups of
4, delta copies), and the roofline kernel name follows the layout code."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

NNZ, M, N = 1200, 100, 90
INFO = {"has": True, "ngroups": 320, "nesc": 5}


def matrix_bytes(prec, code, pass_no=1):
    b = bench.algorithmic_bytes(NNZ, M, N, prec, (INFO, INFO), (code, code))[pass_no - 1]
    c = bench.algorithmic_bytes(NNZ, M, N, prec, None)[pass_no - 1]  # CSR
    return b - c + NNZ * (bench.VAL_BYTES[prec] + 4)


def test_layout_bytes():
    # CSR: value + int32 column per entry
    assert matrix_bytes("f64", 0) == NNZ * 12
    # packed / fused / sliced / tiled: 8-byte index word + 4 values per group, escapes 16 bytes
    for code in (1, 3, 5, 8, 9, 10):
        assert matrix_bytes("q16", code) == 320 * 16 + 5 * 16
        assert matrix_bytes("f64", code) == 320 * 40 + 5 * 16
    # delta copies: 16 bytes per 6 entries (2-byte forms), 4 + 4 values per 4 entries (others)
    for code in (11, 12, 13):
        assert abs(matrix_bytes("q16", code) - NNZ * 16 / 6) < 1e-6
        assert abs(matrix_bytes("f32", code) - NNZ * 20 / 4) < 1e-6
        assert abs(matrix_bytes("f64", code) - NNZ * 36 / 4) < 1e-6
    # tiled step records: 2-byte forms only (the others read code 9's slots)
    assert abs(matrix_bytes("f16", 14) - NNZ * 16 / 6) < 1e-6
    assert matrix_bytes("f32", 14) == 320 * 24 + 5 * 16


def test_kernel_names():
    assert bench.kernel_suffix("f64", 0, False) == "_f64"
    assert bench.kernel_suffix("q16", 0, False) == "_lp"
    assert bench.kernel_suffix("f64", 1, True) == "_pk64"
    assert bench.kernel_suffix("q16", 2, True) == "_pk"
    assert bench.kernel_suffix("q16", 4, True) == "_pkf"
    assert bench.kernel_suffix("f32", 4, True) == "_pk"
    assert bench.kernel_suffix("f64", 6, True) == "_sl"
    assert bench.kernel_suffix("q16", 12, True) == "_dl"

