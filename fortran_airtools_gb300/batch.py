"""Batches of independent SIRT/SART problems (include/fair_batch.h).

No counterpart in the reference, whose ``sirt`` (AIRMs.f90:997-1127) solves one
problem per call: a Batch advances every problem it holds with one kernel
launch per pass and iteration, the iterations captured in a CUDA graph.
Vectors are concatenated over the problems in the order they were added.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._clib import PREC, check, f64, lib, ptr
from .airms import options


class Batch:
    LAYOUTS = {"packed": 0, "tiled": 1, "auto": 2}

    def __init__(self, prec: str = "f32", layout: str = "packed"):
        """layout 'packed' (the packed index streams; CSR in f64), 'tiled'
        (the tiled copies of A and A' for every problem on an N x N image) or
        'auto' (per class of problems the faster of the two, timed on its
        first problem, with the fastest tile shape)."""
        if layout not in self.LAYOUTS:
            raise ValueError("layout must be 'packed', 'tiled' or 'auto'")
        self._h = C.c_void_p()
        check(lib().fair_batch_create(C.byref(self._h), PREC[prec]))
        self.prec = prec
        self.layout = layout
        if layout != "packed":
            check(lib().fair_batch_set_layout(self._h, self.LAYOUTS[layout]))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().fair_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, cuda_stream_ptr: int | None):
        check(lib().fair_batch_set_stream(self._h, cuda_stream_ptr))

    def add(self, A, take: bool = False):
        """Append the matrix of CSRMatrix A (take=True moves it out of A)."""
        check(lib().fair_batch_add(self._h, A.handle, 1 if take else 0))

    def info(self) -> dict:
        np_, m, n, nnz, by = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().fair_batch_info(self._h, C.byref(np_), C.byref(m), C.byref(n), C.byref(nnz),
                                    C.byref(by)))
        return {"problems": np_.value, "rows": m.value, "cols": n.value, "nnz": nnz.value,
                "device_bytes": by.value}

    def problem_layout(self, p: int) -> dict:
        """The layout problem p runs on: {'tiled', 'tile', 'pixel_tile', 'cells'}."""
        v = (C.c_int32 * 4)()
        check(lib().fair_batch_problem_layout(self._h, int(p), v))
        return {"tiled": bool(v[0]), "tile": v[1], "pixel_tile": v[2], "cells": v[3]}

    def pass_bytes(self, sart: bool = True):
        """Algorithmic bytes of the two passes of one iteration."""
        a, b = C.c_int64(), C.c_int64()
        check(lib().fair_batch_pass_bytes(self._h, 1 if sart else 0, C.byref(a), C.byref(b)))
        return a.value, b.value

    def offsets(self):
        k = self.info()["problems"]
        ro, co = np.zeros(k + 1, np.int64), np.zeros(k + 1, np.int64)
        check(lib().fair_batch_offsets(self._h, ptr(ro), ptr(co)))
        return ro, co

    def sirt(self, method: str, b_all, K: int, x0_all=None, opts=None) -> np.ndarray:
        info = self.info()
        b_all, x0_all = f64(b_all), f64(x0_all)
        if b_all.size != info["rows"]:
            raise ValueError("b_all must hold the rows of every problem")
        x = np.empty(info["cols"], np.float64)
        o = opts if opts is not None else options()
        check(lib().fair_batch_sirt(self._h, method.encode(), ptr(b_all), int(K), ptr(x0_all),
                                    C.byref(o), ptr(x)))
        return x

    def prepare(self, method: str, opts=None):
        o = opts if opts is not None else options()
        check(lib().fair_batch_prepare(self._h, method.encode(), C.byref(o)))

    def run_device(self, d_b: int, d_x: int, K: int, batched: bool = True):
        f = lib().fair_batch_run_device if batched else lib().fair_batch_run_device_unbatched
        check(f(self._h, d_b, d_x, int(K)))

    def autotune(self, d_b: int, d_x: int, reps: int = 3):
        cfg = (C.c_int32 * 4)()
        check(lib().fair_batch_autotune(self._h, d_b, d_x, int(reps), cfg))
        return list(cfg)

    def set_config(self, cfg):
        check(lib().fair_batch_set_config(self._h, (C.c_int32 * 4)(*cfg)))
