"""Test inputs (module phantomgallery, phantomgallery.f90) and seeded
synthetic phantoms for the benchmark workloads.

``shepplogan`` is the reference's deterministic 10-ellipse phantom, computed
by the library (phantomgallery.f90:116-164). The reference's random phantoms
draw from the unseeded Fortran stream; the seeded generators here stand in
for them with the shapes the workloads name (a sum of Gaussians, Voronoi
grains, random ellipses, three phases), all on the reference's pixel grid
and vectorised column by column like ``vectorise`` (:672-690).
"""
from __future__ import annotations

import numpy as np

from ._clib import check, lib, ptr


def shepplogan(N: int) -> np.ndarray:
    v = np.empty(N * N, np.float64)
    check(lib().fair_shepplogan(int(N), ptr(v)))
    return v


def phantom(name: str, N: int) -> np.ndarray:
    """choose_phantom (phantomgallery.f90:84-114) evaluated on the GPU:
    'shepplogan', 'smooth', 'grains' (uniform seeds) or '3phases', the random
    ones drawing from the library stream in the reference's order."""
    v = np.empty(N * N, np.float64)
    check(lib().fair_phantom(name.encode(), int(N), ptr(v)))
    return v


def add_white_noise_device(d_b: int, d_bt: int, d_e: int, m: int, eta: float, stream=None):
    """add_white_noise (system_generation.f90:709-745) on device vectors."""
    check(lib().fair_add_white_noise_device(d_bt, d_e, d_b, int(m), float(eta), stream))


def vectorise(img: np.ndarray) -> np.ndarray:
    """Column-major vectorisation (phantomgallery.f90:672-690)."""
    return np.asarray(img, np.float64).reshape(-1, order="F").copy()


def _grid01(N):
    # pixel centres in [0,1]^2: x along columns (left to right), y along rows (top to bottom)
    c = (np.arange(N) + 0.5) / N
    X = np.broadcast_to(c[None, :], (N, N))
    Y = np.broadcast_to(c[::-1][:, None], (N, N))
    return X, Y


def gaussians(N: int, count: int = 20, seed: int = 1) -> np.ndarray:
    """Superposition of `count` Gaussians with centres, widths and amplitudes
    drawn uniformly in [0,1] (image coordinates normalised to [0,1]^2)."""
    rng = np.random.default_rng(seed)
    X, Y = _grid01(N)
    img = np.zeros((N, N))
    for _ in range(count):
        cx, cy, w, a = rng.uniform(0.0, 1.0, 4)
        w = max(w, 1e-3) * 0.25
        img += a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    return vectorise(img)


def grains(N: int, cells: int, seed: int = 2) -> np.ndarray:
    """Voronoi grain image with `cells` cells, values uniform in [0,1]."""
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0.0, 1.0, (cells, 2))
    vals = rng.uniform(0.0, 1.0, cells)
    X, Y = _grid01(N)
    P = np.stack([X.ravel(), Y.ravel()], 1)
    try:  # nearest seed by k-d tree when scipy is present
        from scipy.spatial import cKDTree
        lab = cKDTree(pts).query(P)[1]
    except ImportError:
        best = np.full(P.shape[0], np.inf)
        lab = np.zeros(P.shape[0], np.int64)
        for k in range(cells):
            d = (P[:, 0] - pts[k, 0]) ** 2 + (P[:, 1] - pts[k, 1]) ** 2
            upd = d < best
            best[upd] = d[upd]
            lab[upd] = k
    return vectorise(vals[lab].reshape(N, N))


def random_ellipses(N: int, count: int = 10, seed: int = 3) -> np.ndarray:
    """Sum of `count` random ellipses inside the unit disc, values in [0,1]."""
    rng = np.random.default_rng(seed)
    X, Y = _grid01(N)
    X, Y = 2 * X - 1, 2 * Y - 1
    img = np.zeros((N, N))
    for _ in range(count):
        a, b = rng.uniform(0.05, 0.5, 2)
        x0, y0 = rng.uniform(-0.5, 0.5, 2)
        phi = rng.uniform(0, np.pi)
        amp = rng.uniform(0.1, 1.0)
        u = (X - x0) * np.cos(phi) + (Y - y0) * np.sin(phi)
        w = (Y - y0) * np.cos(phi) - (X - x0) * np.sin(phi)
        img[(u / a) ** 2 + (w / b) ** 2 <= 1.0] += amp
    return vectorise(img / max(img.max(), 1e-12))


def three_phases(N: int, p: int = 100, seed: int = 4) -> np.ndarray:
    """Three-phase image after the recipe of threephases (phantomgallery.f90:201-254):
    two thresholded sums of p bumps at random centres, overlap folded to phase 1."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(1.0, N, N)
    Xc = np.broadcast_to(xs[None, :], (N, N))
    Yc = np.broadcast_to(xs[::-1][:, None], (N, N))
    s = 0.025 * N
    im1 = np.zeros((N, N))
    for cx, cy in rng.uniform(0, 1, (p, 2)) * N:
        im1 += np.exp(-np.abs(Xc - cx) ** 3 / (2.5 * s) ** 3 - np.abs(Yc - cy) ** 3 / (2.5 * s) ** 3)
    im1 = np.where(im1 < 0.35, 0.0, 2.0)
    im2 = np.zeros((N, N))
    for cx, cy in rng.uniform(0, 1, (p, 2)) * N:
        im2 += np.exp(-np.abs(Xc - cx) ** 3 / (2.5 * s) ** 3 - np.abs(Yc - cy) ** 3 / (2.5 * s) ** 3)
    im2 = np.where(im2 < 0.55, 0.0, 1.0)
    x = im1 + im2
    x[x == 3.0] = 1.0
    return vectorise(x / max(x.max(), 1e-12))


__all__ = ["shepplogan", "vectorise", "gaussians", "grains", "random_ellipses", "three_phases"]
