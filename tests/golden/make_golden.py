"""Generate the golden fixtures in tests/golden/ from the CPU oracle.

python tests/golden/make_golden.py

The fixtures are small: system matrices of a few problems that exercise the
special cases of the ray tracer (axis-aligned and diagonal rays, rays on grid
lines, the odd-p fan angles), their transposes, and short SIRT / ART runs.
They pin the oracle against regressions and give the GPU tests committed
vectors to compare with.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def cases():
    th_par = np.concatenate([[0.0, np.pi / 4, np.pi / 2], O.linspace(0.2, 2.9, 5)])
    yield "par_16_8_24", dict(kind="parallel", n=16, nth=8, p=24, theta=th_par)
    yield "par_16_3_15", dict(kind="parallel", n=16, nth=3, p=15, theta=np.array([0.0, 0.5, np.pi / 4]))
    th_fan = 2 * np.pi * np.arange(12) / 12
    yield "fan_16_12_17", dict(kind="fan", n=16, nth=12, p=17, r=2.0, dw=17 / 16, sd=2.0,
                               theta=th_fan, fix=False)
    yield "fan_16_12_17_fix", dict(kind="fan", n=16, nth=12, p=17, r=2.0, dw=17 / 16, sd=2.0,
                                   theta=th_fan, fix=True)
    yield "fan_15_12_18", dict(kind="fan", n=15, nth=12, p=18, r=1.5, dw=1.2, sd=2.5,
                               theta=th_fan, fix=False)


def build(c):
    if c["kind"] == "parallel":
        return O.paralleltomo(c["n"], c["nth"], c["p"], c["theta"])
    return O.fanlineartomo(c["n"], c["nth"], c["p"], c["r"], c["dw"], c["sd"], c["theta"],
                           geometry_fix=c["fix"])


def solve(R, n):
    xt = O.shepplogan(n)
    b = O.matvecmul(R, xt)
    out = {"b": b}
    out["sirt_cimmino"] = O.sirt("cimmino", R, b, 10, opts=O.options(relaxpar=1.5, lbound=0.0))
    out["sirt_sart"] = O.sirt("sart", R, b, 10, opts=O.options(lbound=0.0, ubound=1.0))
    out["kaczmarz"] = O.art("kaczmarz", R, b, [2], opts=O.options(relaxpar=0.25))[:, 0]
    out["symkaczmarz"] = O.art("symkaczmarz", R, b, [2], opts=O.options(relaxpar=0.5, lbound=0.0))[:, 0]
    return out


def main():
    for name, c in cases():
        R = build(c)
        T = O.reorder(R)
        arrays = dict(IA=R.IA, JA=R.JA, vA=R.vA, m=R.m, n=R.n, TIA=T.IA, TJA=T.JA, TvA=T.vA,
                      theta=c["theta"])
        arrays.update(solve(R, c["n"]))
        meta = {k: v for k, v in c.items() if k != "theta"}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(repr(meta)), **arrays)
        print(name, R.m, R.n, R.nnz)


if __name__ == "__main__":
    main()
