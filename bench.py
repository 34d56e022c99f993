#!/usr/bin/env python
"""SIRT iterations/s on the parallel-beam N=1024 problem (720 angles over
[0, pi), 1448 bins; ~9.6e8 nonzeros) -- one JSON line on stdout.

A step is one SIRT (Cimmino) iteration: a residual pass over A and a
backprojection/update pass over A'. ``value`` is iterations/s with the matrix
and vectors resident in HBM (CUDA events on the launching stream); ``e2e`` is
the same metric through the host C-ABI call fair_sirt (host b in, host x
out, copies inside the timed region); ``forms`` gives the FP64, FP32 and
16-bit forms with their error against the oracle's FP64 iterate (and the GPU
FP64 one); ``roofline`` is the dominant kernel's algorithmic bytes over its
average launch time against the measured HBM copy bandwidth; ``cpu_baseline``
is the CPU oracle (a restatement of the reference's Fortran) on a bounded
sample of the same iteration, three ways; ``secondary`` holds the lines of
the other workloads (Kaczmarz family, adjoint, batch, matrix-free and stored
FP32 at N=2048), each run in its own process after the headline.

--impl reference times the CPU restatement of the reference (oracle/, all
host threads for the row-parallel product and for the transposed product, the
latter race-free with per-thread copies) on the same workload, one bounded
sample of the iteration per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, NTH, P = 1024, 720, 1448
METRIC = "SIRT iter/s at N=1024 (FP64 vs mixed, <=1e-5 rel err); SpMV GB/s vs HBM peak"
WORKLOAD = "parallel-beam N=1024, 720 angles over [0,pi), 1448 bins; SIRT (Cimmino)"
PREC_NAMES = {"f64": 0, "f32": 1, "f16": 2, "q16": 3}
VAL_BYTES = {"f64": 8, "f32": 4, "f16": 2, "q16": 2}


def theta():
    return np.pi * np.arange(NTH) / NTH


def noisy(b, eta=0.01, seed=1):
    """b + e with e Gaussian (seeded), scaled to ||e|| = eta ||b|| (the scaling
    of add_white_noise). The reference's Newton inverse-CDF cannot always meet
    its 1e-14 tolerance in the upper tail on aarch64's libm, so the synthetic
    benchmark inputs draw their normals with numpy instead."""
    e = np.random.default_rng(seed).standard_normal(b.size)
    e *= eta * np.linalg.norm(b) / np.linalg.norm(e)
    return b + e


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


def dist_init(world, backend):
    """One process per GPU (torchrun): the process group for the barrier and the
    max-over-ranks time; replicas exchange nothing else."""
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world, device):
    """The slowest rank's value (times are taken as the max over ranks)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sm_count(torch, device):
    return torch.cuda.get_device_properties(device).multi_processor_count


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(nnz, m, n, prec, packed=None, codes=(0, 0)):
    """Bytes each SIRT pass must move once (matrix streamed, vectors once).
    `packed` = (info of A, info of A') when the pass reads a layout built on
    the packed index stream, `codes` the passes' layout codes. Per group of 4
    entries: 8 bytes of index + 4 values (packed stream, fused records,
    sliced and tiled copies; 16 bytes per escaped group); delta copies: 4
    bytes of steps + 4 values per 4 entries (FP32, FP64), 16 bytes per 6
    entries (2-byte forms, also the tiled step records of code 14)."""
    sv = VAL_BYTES[prec]
    sx = 8 if prec == "f64" else 4
    two = prec in ("f16", "q16")

    def matrix(info, code):
        if info is None or not info["has"] or code == 0:
            return nnz * (sv + 4)
        if (11 <= code <= 13) or (code == 14 and two):
            return nnz * 16 / 6 if two else nnz * (4 + 4 * sv) / 4
        return info["ngroups"] * (8 + 4 * sv) + info["nesc"] * 16

    pa, pt = packed if packed else (None, None)
    pass1 = matrix(pa, codes[0]) + (m + 1) * 8 + n * sx + m * 8 + m * 8 + m * sx
    pass2 = matrix(pt, codes[1]) + (n + 1) * 8 + m * sx + 2 * n * 8 + (0 if prec == "f64" else n * 4)
    return pass1, pass2


def kernel_suffix(prec, code, on_pk):
    """Name suffix of the SIRT pass kernel that layout `code` runs (layout
    codes of fair_sirt_set_lanes)."""
    if not on_pk:
        return "_f64" if prec == "f64" else "_lp"
    if 11 <= code <= 13:
        return "_dl"
    if code >= 5:
        return "_sl"
    if prec == "f64":
        return "_pk64"
    return "_pkf" if code >= 3 and prec in ("f16", "q16") else "_pk"


def traffic_from_profiles(kernel, prec, nnz):
    """Per-launch DRAM bytes of `kernel` in form `prec` from the ncu capture
    summarised in profiles/ (recorded for the N=1024 launch), if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f).get(prec, {}).get(kernel)
        return None if t is None or nnz != 961254632 else t
    except Exception:
        return None


# --------------------------------------------------------------- CPU timing ----
def workload_config(m, n, nnz):
    """The `config` of both arms (the same keys and values for the same workload)."""
    return {"workload": WORKLOAD, "n": N, "angles": NTH, "bins": P, "m": m, "ncols": n,
            "nnz": nnz, "method": "cimmino", "precision": "f64",
            "l2": "inputs larger than L2 (FP64 matrix %.1f GB per pass)" % (nnz * 12 / 1e9)}


def cpu_sirt_rate(O, R, b, budget_s, nthreads, steps=None, warmup=0, mode="racefree"):
    """Time the oracle's SIRT iteration (Cimmino) on a contiguous block of
    angles of R sized to `budget_s`; returns (iterations/s of the full
    problem, description, seconds per sample step). `mode` is the threaded
    transposed product: 'racefree' (per-thread copies added in thread order)
    or 'racy' (the reference's shared scatter, sparse_matrices.f90:382-392)."""
    m, p = R.m, P
    O.set_mmcs_mode(mode)

    # trial on ~1% of the angles to size the sample
    def sub(nang):
        r1 = nang * p
        IA = R.IA[: r1 + 1].copy()
        nz = int(IA[-1])
        S = O.OracleCSR(r1, R.n, IA, R.JA[:nz], R.vA[:nz])
        return S, b[:r1], nz

    try:
        S, bs, nz = sub(max(1, NTH // 100))
        t0 = time.perf_counter(); O.sirt("cimmino", S, bs, 0, nthreads=nthreads)
        t1 = time.perf_counter(); O.sirt("cimmino", S, bs, 1, nthreads=nthreads)
        t2 = time.perf_counter()
        per_nnz = max((t2 - t1) - (t1 - t0), 1e-9) / max(nz, 1)
        k = steps if steps else 3
        nang = int(min(NTH, max(1, budget_s / (per_nnz * R.nnz / NTH) / (k + warmup))))
        S, bs, nz = sub(nang)
        if warmup:
            O.sirt("cimmino", S, bs, warmup, nthreads=nthreads)
        t0 = time.perf_counter(); O.sirt("cimmino", S, bs, 0, nthreads=nthreads)
        t1 = time.perf_counter(); O.sirt("cimmino", S, bs, k, nthreads=nthreads)
        t2 = time.perf_counter()
    finally:
        O.set_mmcs_mode("racefree")
    step = ((t2 - t1) - (t1 - t0)) / k
    frac = nz / R.nnz
    rate = frac / step
    desc = (f"SIRT (Cimmino) iteration restricted to the first {nang} of {NTH} angles "
            f"({frac:.3f} of the nonzeros), {k} iterations, scaled to full iterations")
    return rate, desc, step


def cpu_variants(O, R, b, budget_s, nthreads):
    """The reference's CPU iteration three ways on the machine's host cores: the
    row-parallel product with the transposed product on all threads made
    race-free (the headline CPU figure: the fastest correct form), the same
    with the transposed product as the reference ships it (a shared scatter
    with no atomics: racy, updates are lost; its error is one full-size
    product against the serial one), and everything on one thread."""
    out = {}
    r, d, _ = cpu_sirt_rate(O, R, b, budget_s, nthreads)
    out["racefree_all_threads"] = {"value": r, "unit": "iter/s", "cores": nthreads, "sample": d}
    r, d, _ = cpu_sirt_rate(O, R, b, budget_s, nthreads, mode="racy")
    y = np.random.default_rng(7).random(R.m)
    w_serial = O.transvecmul(R, y)
    w_racy = O.transvecmul_racy(R, y, nthreads)
    err = float(np.linalg.norm(w_racy - w_serial) / np.linalg.norm(w_serial))
    out["racy_all_threads"] = {"value": r, "unit": "iter/s", "cores": nthreads, "sample": d,
                               "label": "racy: the shipped shared scatter of MMCS",
                               "rel_err_one_product_vs_serial": err}
    r, d, _ = cpu_sirt_rate(O, R, b, budget_s, 1)
    out["one_thread"] = {"value": r, "unit": "iter/s", "cores": 1, "sample": d}
    return out


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from oracle import oracle as O
    from fortran_airtools_gb300 import phantomgallery as pg  # numpy-only generators
    nthreads = os.cpu_count() or 1
    th = theta()
    R = O.paralleltomo_mt(N, NTH, P, th, nthreads)
    xt = pg.gaussians(N, 20, seed=1)
    b = O.matvecmul(R, xt, nthreads=nthreads)
    bt = noisy(b)
    budget = float(os.environ.get("FAIR_REF_BUDGET_S", "60"))
    rate, desc, step = cpu_sirt_rate(O, R, bt, budget, nthreads, steps=args.steps,
                                     warmup=args.warmup)
    variants = None
    if not args.no_cpu:
        variants = cpu_variants(O, R, bt, float(os.environ.get("FAIR_CPU_BUDGET_S", "8")),
                                nthreads)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "iter/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded 20-Gaussian phantom, 1% noise)",
            "config": workload_config(R.m, R.n, R.nnz),
            "cpu_baseline": {"value": rate, "unit": "iter/s", "cores": nthreads, "kind": "port",
                             "sample": desc + "; transposed product race-free on all threads",
                             "variants": variants},
            "e2e": {"value": rate, "unit": "iter/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------- GPU arm ----
def run_ours(args):
    import ctypes as C

    import torch

    import fortran_airtools_gb300 as F
    from fortran_airtools_gb300._clib import check, lib

    rank, world, local = env_rank()
    dist_init(world, "nccl")
    torch.cuda.set_device(local)
    L = lib()

    def barrier():
        dist_barrier(world)

    stream = torch.cuda.Stream()
    th = theta()
    t0 = time.perf_counter()
    A = F.paralleltomo(F.Data(n=N, p=P, nth=NTH, theta=th))
    build_s = time.perf_counter() - t0
    A.set_stream(stream.cuda_stream)
    m, n, nnz = A.info()
    xt = F.phantomgallery.gaussians(N, 20, seed=1)
    b = A.matvecmul(xt)
    bt = noisy(b)
    d_b = torch.from_numpy(bt).to(f"cuda:{local}")
    d_x = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
    opts = F.airms.options()  # reference defaults: relaxpar 1, no bounds
    h = A.handle

    forms = {}
    results = {}
    results_or = {}  # the iterate after k_or iterations, compared with the oracle's
    k_or = max(1, min(args.steps, 20))
    packed = {}
    form_list = ["f64"] + [f for f in args.forms.split(",") if f and f != "f64"]
    if args.prec not in form_list:
        form_list.append(args.prec)
    for prec in form_list:
        A.set_precision(prec)
        check(L.fair_sirt_prepare(h, b"cimmino", C.byref(opts)))
        cfg = (C.c_int32 * 4)(8, 8, *((0, 0) if prec == "f64" else (1, 1)))  # library defaults
        if args.lanes:  # fixed lanes per row (and groups per lane) of the two passes
            v = [int(t) for t in args.lanes.split(",")]
            cfg[:] = (v + [1, 1])[:4] if len(v) == 2 else v[:4]
            check(L.fair_sirt_set_lanes(h, cfg))
        elif not args.no_tune:  # fastest lanes per row / groups per lane of each pass
            check(L.fair_sirt_autotune(h, d_b.data_ptr(), d_x.data_ptr(), 3, cfg))
        with torch.cuda.stream(stream):
            d_x.zero_()
            check(L.fair_sirt_run_device(h, d_b.data_ptr(), d_x.data_ptr(), args.warmup))
            d_x.zero_()
        stream.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sampler = ClockSampler(local) if prec == args.prec else None
        if sampler:
            sampler.start()
        torch.cuda.synchronize()
        e0.record(stream)
        check(L.fair_sirt_run_device(h, d_b.data_ptr(), d_x.data_ptr(), args.steps))
        e1.record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        ms = max_over_ranks(e0.elapsed_time(e1), world, f"cuda:{local}")
        results[prec] = d_x.cpu().numpy()
        if k_or == args.steps:
            results_or[prec] = results[prec]
        else:  # outside the timed region
            with torch.cuda.stream(stream):
                d_x.zero_()
            check(L.fair_sirt_run_device(h, d_b.data_ptr(), d_x.data_ptr(), k_or))
            stream.synchronize()
            results_or[prec] = d_x.cpu().numpy()
        # per-pass launch durations (CUDA events around each kernel)
        ms1, ms2 = C.c_float(), C.c_float()
        with torch.cuda.stream(stream):
            d_x.zero_()
        stream.synchronize()
        kt = max(3, min(args.steps, 20))
        check(L.fair_sirt_run_device_timed(h, d_b.data_ptr(), d_x.data_ptr(), kt,
                                           C.byref(ms1), C.byref(ms2)))
        launches = C.c_int64()
        check(L.fair_sirt_launches(h, args.steps, C.byref(launches)))
        forms[prec] = {"iter_per_s": world * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                       "pass1_ms": ms1.value / kt, "pass2_ms": ms2.value / kt,
                       "launches": launches.value, "clocks": clocks,
                       "pass_config": None if args.no_tune and not args.lanes else
                       {"lanes_per_row": [cfg[0], cfg[1]], "groups_per_lane": [cfg[2], cfg[3]]}}
        # the passes that read the packed stream (groups per lane > 0)
        pk = (A.packed_info(), A.packed_info(transposed=True))
        use = [pk[i]["has"] and cfg[2 + i] > 0 for i in (0, 1)]
        if any(use):
            packed[prec] = tuple(pk[i] if use[i] else None for i in (0, 1))
            forms[prec]["packed_index"] = {"A": pk[0] if use[0] else None,
                                           "AT": pk[1] if use[1] else None}
    for prec in form_list[1:]:
        r = results["f64"]
        forms[prec]["rel_err_vs_f64"] = float(np.linalg.norm(results[prec] - r) / np.linalg.norm(r))

    hp = args.prec
    head = forms[hp]
    peak, peak_kind = hbm_peak()
    def pass_codes(prec):
        pc = forms[prec].get("pass_config")
        if pc:
            return tuple(pc["groups_per_lane"])
        return (0, 0) if prec == "f64" else (1, 1)  # the library's default layouts

    b1, b2 = algorithmic_bytes(nnz, m, n, hp, packed.get(hp), pass_codes(hp))
    dom = 2 if head["pass2_ms"] >= head["pass1_ms"] else 1
    pk = packed.get(hp)
    on_pk = bool(pk and pk[dom - 1])
    code = (head["pass_config"]["groups_per_lane"][dom - 1] if head.get("pass_config")
            else 0 if hp == "f64" else 1)  # the library's default layouts
    kname = ("k_tl_partials" if code in (9, 10, 14) and on_pk else
             {1: "k_sirt_resid", 2: "k_sirt_update"}[dom] + kernel_suffix(hp, code, on_pk))
    dom_bytes = b2 if dom == 2 else b1
    dom_ms = head["pass2_ms"] if dom == 2 else head["pass1_ms"]
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    fp64_pipe = None
    if hp == "f64":
        # the FP64 form is bound by the FP64 pipe: one multiply-add per nonzero
        # against 2 FP64 lanes per clock per SM at the sampled SM clock
        mhz = (head.get("clocks") or {}).get("sm_mhz") or 2070.0
        dpeak = 2 * sm_count(torch, local) * mhz * 1e6
        fp64_pipe = {"achieved_dfma_per_s": nnz / (dom_ms / 1e3), "peak_dfma_per_s": dpeak,
                     "frac": nnz / (dom_ms / 1e3) / dpeak,
                     "peak_basis": "2 FP64 lanes/clock/SM x SMs x median sampled SM clock"}
    traffic = traffic_from_profiles(kname, hp, nnz)
    for prec in forms:
        p1, p2 = algorithmic_bytes(nnz, m, n, prec, packed.get(prec), pass_codes(prec))
        f = forms[prec]
        f["iteration_gbs"] = (p1 + p2) / (f["ms_per_step"] / 1e3) / 1e9
        f["iteration_frac_of_hbm"] = f["iteration_gbs"] / peak

    # e2e through the host C-ABI (host b in, host x out)
    A.set_precision(hp)
    F.airms.sirt("cimmino", A, bt, max(1, args.warmup), opts=opts)
    barrier()
    t0 = time.perf_counter()
    F.airms.sirt("cimmino", A, bt, args.steps, opts=opts)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, f"cuda:{local}")

    # the oracle (outside every timed region): its own matrix, compared with
    # the GPU's, and its FP64 iterate after k_or iterations, against which
    # every form's iterate is reported
    cpu = None
    oracle_check = None
    if rank == 0 and world == 1 and not args.no_oracle:
        from oracle import oracle as O
        nthreads = os.cpu_count() or 1
        t0 = time.perf_counter()
        R = O.paralleltomo_mt(N, NTH, P, th, nthreads)
        ob_s = time.perf_counter() - t0
        vA, IA, JA = A.arrays()
        same = bool(np.array_equal(IA, R.IA) and np.array_equal(JA, R.JA))
        vrel = (float(np.max(np.abs(vA - R.vA) / np.maximum(np.abs(R.vA), 1e-300)))
                if same and R.nnz else None)
        del vA, IA, JA
        xo = O.sirt("cimmino", R, bt, k_or, nthreads=nthreads)
        no = np.linalg.norm(xo)
        for prec in forms:
            forms[prec]["rel_err_vs_oracle"] = float(np.linalg.norm(results_or[prec] - xo) / no)
            forms[prec]["oracle_iterations"] = k_or
        oracle_check = {"matrix_ia_ja_equal": same, "matrix_va_max_rel_diff": vrel,
                        "iterations": k_or, "oracle_build_s": ob_s, "threads": nthreads,
                        "note": "oracle FP64 Cimmino iterate after `iterations` steps from x = 0, "
                                "on the oracle's own matrix, vs each form's GPU iterate"}
        if not args.no_cpu:
            var = cpu_variants(O, R, bt, float(os.environ.get("FAIR_CPU_BUDGET_S", "8")), nthreads)
            head_cpu = var["racefree_all_threads"]
            cpu = {"value": head_cpu["value"], "unit": "iter/s", "cores": nthreads, "kind": "port",
                   "sample": head_cpu["sample"] + "; transposed product race-free on all threads",
                   "variants": var}
        del R

    if rank == 0:
        line = {
            "metric": METRIC, "value": head["iter_per_s"], "unit": "iter/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": hp, "data": "synthetic (seeded 20-Gaussian phantom, 1% noise)",
            "config": workload_config(m, n, nnz),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "geometry_build_s": build_s,
            "oracle_check": oracle_check,
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "algorithmic_bytes_per_launch": dom_bytes,
                         "traffic": traffic,
                         "limiter": "fp64 pipe" if fp64_pipe else "hbm / load latency",
                         "fp64_pipe": fp64_pipe},
            "forms": forms,
            "e2e": {"value": world * args.steps / e2e_s, "unit": "iter/s",
                    "h2d_bytes_per_step": 8 * m / args.steps,
                    "d2h_bytes_per_step": 8 * n / args.steps,
                    "note": "one fair_sirt call of `steps` iterations: b uploaded, x downloaded"},
            "gpu_launches": head["launches"],
            "clocks": head["clocks"],
            "cpu_baseline": cpu,
        }
    A.close()
    if rank == 0:
        if world == 1 and not args.no_secondary:
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            line["secondary"] = run_secondary(args)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


SECONDARY = [  # (name, extra arguments, time limit in s): the other workloads of the path
    ("c1_cimmino", ["--workload", "c1"], 300),
    ("kaczmarz", ["--workload", "kaczmarz", "--no-cpu"], 300),
    ("adjoint", ["--workload", "adjoint", "--no-cpu"], 300),
    ("batch", ["--workload", "batch", "--batch-layout", "auto", "--no-cpu"], 600),
    ("mfree", ["--workload", "mfree", "--mf-sizes", "2048,fan"], 600),
]


def run_secondary(args):
    """The secondary workloads (the fan N=128 Cimmino run, Kaczmarz family,
    adjoint, batch, matrix-free and stored FP32 at N=2048), each in a process
    of its own after the headline run has freed its GPU memory; their JSON
    lines are collected here so that one bench run records every workload.
    CPU baselines are skipped but for the Cimmino run (a few seconds; the
    headline line carries the main CPU comparison)."""
    out = {}
    for name, extra, limit in SECONDARY:
        t0 = time.perf_counter()
        try:
            r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + extra,
                               capture_output=True, text=True, timeout=limit, cwd=ROOT)
            lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
            out[name] = {"rc": r.returncode, "wall_s": time.perf_counter() - t0, "lines": lines}
            if r.returncode != 0:
                out[name]["stderr_tail"] = r.stderr[-600:]
        except subprocess.TimeoutExpired:
            out[name] = {"rc": None, "error": f"timed out after {limit} s"}
    return out


def run_c1(args):
    """The Cimmino run of the plain FP64 configuration (a secondary line): fan
    beam N=128, 360 angles over [0, 2pi), 181 unit bins, source radius 2N,
    Shepp-Logan phantom, 1% noise (seed 0), Cimmino SIRT for 100 iterations
    with relaxation 1.9/||M^(-1/2) A||^2 (M the Cimmino row weights; the norm
    by power iteration on the host) and lower bound 0, FP64. Iterations/s through the host
    call (b uploaded, x downloaded, the weights computed inside the call as the
    reference does per call), beside the oracle's Cimmino on one core and on
    all host threads (CPU time of the same 100 iterations), and the GPU
    iterate's error against the oracle's."""
    import fortran_airtools_gb300 as F
    from oracle import oracle as O
    n, nth, p, K = 128, 360, 181, 100
    th = 2 * np.pi * np.arange(nth) / nth
    d = F.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th)
    A = F.fanlineartomo(d)
    m, ncol, nnz = A.info()
    b = noisy(A.matvecmul(F.phantomgallery.shepplogan(n)), seed=0)
    # relaxation 1.9 / sigma_max(M^(-1/2) A)^2, M = m ||a_i||^2 (Cimmino's weights)
    import scipy.sparse as sp
    vA, IA, JA = A.arrays()
    S = sp.csr_matrix((vA, JA - 1, IA), shape=(m, ncol))
    nr = np.sqrt(np.asarray(S.multiply(S).sum(axis=1)).ravel())
    B = sp.diags(np.where(nr > 0, 1.0 / np.sqrt(m * nr * nr + (nr == 0)), 0.0)) @ S
    v = np.random.default_rng(0).uniform(size=ncol)
    for _ in range(200):
        v = B.T @ (B @ v)
        v /= np.linalg.norm(v)
    lam = 1.9 / np.linalg.norm(B @ v) ** 2
    opts = F.airms.options(relaxpar=lam, lbound=0.0)
    F.airms.sirt("cimmino", A, b, [K], opts=opts)  # warm-up
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        x = F.airms.sirt("cimmino", A, b, [K], opts=opts)
    gpu_s = (time.perf_counter() - t0) / reps
    R = O.OracleCSR(m, ncol, IA, JA, vA)
    ro = O.options(relaxpar=lam, lbound=0.0)
    nthreads = os.cpu_count() or 1
    cpu = {}
    xo = None
    for label, nt in (("one_thread", 1), ("all_threads", nthreads)):
        if args.no_cpu and label == "one_thread":
            continue
        t0 = time.perf_counter()
        xo = O.sirt("cimmino", R, b, K, opts=ro, nthreads=nt)
        cpu[label] = {"value": K / (time.perf_counter() - t0), "unit": "iter/s", "cores": nt}
    head = cpu.get("one_thread", cpu["all_threads"])
    line = {"metric": "cimmino iter/s (100 iterations)", "workload": f"fan N={n}, {nth} angles, {p} bins",
            "value": K / gpu_s, "unit": "iter/s", "ms_per_call": gpu_s * 1e3, "iterations": K,
            "relaxpar": lam,
            "nnz": nnz, "dtype": "f64", "rel_err_vs_oracle": float(np.linalg.norm(x - xo) / np.linalg.norm(xo)),
            "note": "fair_sirt host call: b uploaded, x downloaded, weights computed in the call",
            "cpu_baseline": {"value": head["value"], "unit": "iter/s", "cores": head["cores"], "kind": "port",
                             "sample": f"{K} iterations of the same problem", "variants": cpu}}
    print(json.dumps(line), flush=True)
    A.close()
    return 0


def run_kaczmarz(args):
    """Kaczmarz family (a secondary measurement, one JSON line per case):
    fan beam N=512, 720 angles over [0, 2pi), 725 unit bins, R = 2N, three-phase
    phantom, bounds [0,1], FP64, 20 sweeps: random Kaczmarz with row-norm
    probabilities and symmetric Kaczmarz; and fan beam N=128, 360 angles, 181
    bins, 10 natural-order sweeps with relaxation 0.25. Rows/s and sweeps/s
    through the host C-ABI call (b in, x out; the call's level schedules are
    built inside it), beside the oracle's serial sweep on one core (the
    reference's sweep is serial)."""
    import fortran_airtools_gb300 as F
    from oracle import oracle as O
    cases = [
        ("randkaczmarz", dict(n=512, nth=720, p=725), dict(rowprobability=True, lbound=0.0, ubound=1.0), 20),
        ("symkaczmarz", dict(n=512, nth=720, p=725), dict(lbound=0.0, ubound=1.0), 20),
        ("kaczmarz", dict(n=128, nth=360, p=181), dict(relaxpar=0.25), 10),
    ]
    if args.kacz_cases:
        cases = [c for c in cases if c[0] in args.kacz_cases.split(",")]
    for method, g, o, sweeps in cases:
        th = 2 * np.pi * np.arange(g["nth"]) / g["nth"]
        d = F.Data(n=g["n"], p=g["p"], nth=g["nth"], r=2.0, dw=g["p"] / g["n"], sd=2.0, theta=th)
        A = F.fanlineartomo(d)
        m, n, nnz = A.info()
        xt = F.phantomgallery.three_phases(g["n"], seed=4) if g["n"] == 512 else \
            F.phantomgallery.shepplogan(g["n"])
        b = noisy(A.matvecmul(xt), seed=4)
        opts = F.airms.options(**o)
        nrow = int(np.count_nonzero(A.row_norms(2)))
        F.airms.random_seed(4)
        F.airms.art(method, A, b, [2 if method == "symkaczmarz" else 1], opts=opts)  # warm-up
        F.airms.random_seed(4)
        t0 = time.perf_counter()
        F.airms.art(method, A, b, [sweeps], opts=opts)
        gpu_s = time.perf_counter() - t0
        rows = nrow * sweeps  # row projections (symkaczmarz: K counts single sweeps)
        cpu = None
        if not args.no_cpu:
            vA, IA, JA = A.arrays()
            R = O.OracleCSR(m, n, IA, JA, vA)
            ro = O.options(**o)
            O.random_seed(4)
            k = 2 if method == "symkaczmarz" else 1
            t0 = time.perf_counter()
            O.art(method, R, b, [k], opts=ro)
            cpu_s = (time.perf_counter() - t0) / k
            cpu = {"value": nrow / cpu_s, "unit": "rows/s", "cores": 1, "kind": "port",
                   "sample": f"{k} sweep(s) of the same problem"}
        line = {"metric": f"{method} rows/s", "workload": f"fan N={g['n']}, {g['nth']} angles, {g['p']} bins",
                "value": rows / gpu_s, "unit": "rows/s", "sweeps_per_s": sweeps / gpu_s,
                "sweeps": sweeps, "nonzero_rows": nrow, "nnz": nnz, "dtype": "f64",
                "note": "fair_art host call: b uploaded, x downloaded", "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
        A.close()
    return 0


def run_adjoint(args):
    """Differentiation workload (secondary lines): 16 parallel-beam problems
    N=256, 360 angles over [0, pi), 362 bins sharing one matrix, random-ellipse
    phantoms (seed 3), K=20 SIRT steps with the nonnegativity projection, loss
    0.5 ||x_K - x_true||^2; one fair_sirt_adjoint call returns x_K and the
    gradients for all 16 problems. FP64 and FP32, beside the oracle's FP64
    adjoint of one problem on one core scaled to 16."""
    import fortran_airtools_gb300 as F
    from oracle import oracle as O
    n, nth, p, K, nb = 256, 360, 362, 20, 16
    th = np.pi * np.arange(nth) / nth
    A = F.paralleltomo(F.Data(n=n, p=p, nth=nth, theta=th))
    m = A.m
    X = np.stack([F.phantomgallery.random_ellipses(n, seed=3 + s) for s in range(nb)], 1)
    B = np.stack([noisy(A.matvecmul(X[:, c]), seed=3 + c) for c in range(nb)], 1)
    lam = np.full(nb, 1.5)
    o = F.airms.options(lbound=0.0)
    cpu = None
    for prec in ("f64", "f32"):
        A.set_precision(prec)
        xK, _, _, _ = F.airms.sirt_adjoint("cimmino", A, B, K, lam, np.zeros((A.n, nb)), opts=o)
        GX = xK - X
        F.airms.sirt_adjoint("cimmino", A, B, K, lam, GX, opts=o)  # warm-up
        t0 = time.perf_counter()
        F.airms.sirt_adjoint("cimmino", A, B, K, lam, GX, opts=o)
        dt = time.perf_counter() - t0
        if cpu is None and not args.no_cpu:
            vA, IA, JA = A.arrays()
            R = O.OracleCSR(m, A.n, IA, JA, vA)
            t0 = time.perf_counter()
            O.sirt_adjoint("cimmino", R, B[:, 0], K, 1.5, GX[:, 0], opts=O.options(lbound=0.0))
            c1 = time.perf_counter() - t0
            cpu = {"value": 1.0 / (c1 * nb), "unit": "batch gradients/s", "cores": 1,
                   "kind": "port", "sample": "one problem's FP64 adjoint, scaled to 16 problems"}
        print(json.dumps({"metric": "adjoint of K=20 SIRT steps, 16 problems", "value": 1.0 / dt,
                          "unit": "batch gradients/s", "ms_per_batch": dt * 1e3,
                          "workload": f"parallel N={n}, {nth} angles, {p} bins, 16 right-hand sides",
                          "dtype": prec, "nnz": A.nnz, "cpu_baseline": cpu,
                          "note": "fair_sirt_adjoint host call: forward with sqrt(K) checkpoints, "
                                  "recomputation and reverse sweep"}), flush=True)
    A.close()
    return 0


def run_batch(args):
    """Batched SART (a secondary line): heterogeneous fan-beam problems, seed 2:
    N uniform on {64, 96, ..., 512}, angles uniform on 90..720 over [0, 2pi),
    p = ceil(1.42 N) unit bins, source at R = 2N, detector at 2N; Voronoi
    grain phantoms with 50-400 cells and values uniform in [0,1]; 0.5% seeded
    noise; SART, 50 iterations, box [0,1], FP32 values with FP64 weights, on
    each layout of --batch-layout (one line each): 'tiled', the tiled copies
    of A and A' (two launches per pass for the whole batch: partial sums, row
    sums), and 'packed', the packed index streams (one launch per pass). The
    50 iterations are replayed from one CUDA graph; the same iterations
    launched problem by problem are timed beside it, and the oracle's serial
    SART on a sample of the problems, scaled by nonzeros, gives the CPU
    baseline."""
    for layout in [t for t in args.batch_layout.split(",") if t]:
        run_batch_layout(args, layout)
    return 0


def run_batch_layout(args, layout):
    import ctypes as C
    import math

    import torch

    import fortran_airtools_gb300 as F
    from fortran_airtools_gb300._clib import check, lib
    from oracle import oracle as O
    K = 50
    nprob = args.batch_problems
    rng = np.random.default_rng(2)
    Ns = rng.choice(np.arange(64, 513, 32), nprob)
    nths = rng.integers(90, 721, nprob)
    cells = rng.integers(50, 401, nprob)
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    B = F.Batch(args.batch_prec, layout=layout)
    bs, samples = [], []
    t0 = time.perf_counter()
    for i in range(nprob):
        n, nth = int(Ns[i]), int(nths[i])
        p = int(math.ceil(1.42 * n))
        th = 2 * np.pi * np.arange(nth) / nth
        A = F.fanlineartomo(F.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
        x = F.phantomgallery.grains(n, int(cells[i]), seed=1000 + i)
        b = noisy(A.matvecmul(x), eta=0.005, seed=1000 + i)
        bs.append(b)
        if not args.no_cpu and len(samples) < 3 and n <= 160:
            m_, n_, _ = A.info()
            vA, IA, JA = A.arrays()
            samples.append((O.OracleCSR(m_, n_, IA, JA, vA), b))
        B.add(A, take=True)
        A.close()
    build_s = time.perf_counter() - t0
    info = B.info()
    ball = np.concatenate(bs)
    shapes = {}
    for i in range(nprob):  # the layout each problem runs on
        lay = B.problem_layout(i)
        key = (f"tiled {lay['tile']}/{lay['pixel_tile']}x{lay['cells']}" if lay["tiled"]
               else "packed")
        shapes[key] = shapes.get(key, 0) + 1
    B.set_stream(stream.cuda_stream)
    opts = F.airms.options(lbound=0.0, ubound=1.0)
    B.prepare("sart", opts)
    d_b = torch.from_numpy(ball).cuda()
    d_x = torch.zeros(info["cols"], dtype=torch.float64, device="cuda")
    cfg = None
    if not args.no_tune:
        cfg = B.autotune(d_b.data_ptr(), d_x.data_ptr(), 3)

    def timed(batched):
        with torch.cuda.stream(stream):
            d_x.zero_()
        B.run_device(d_b.data_ptr(), d_x.data_ptr(), K, batched=batched)  # warm-up (and capture)
        stream.synchronize()
        with torch.cuda.stream(stream):
            d_x.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        B.run_device(d_b.data_ptr(), d_x.data_ptr(), K, batched=batched)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1)

    sampler = ClockSampler(0)
    sampler.start()
    ms_b = timed(True)
    clocks = sampler.stop()
    xb = d_x.cpu().numpy()
    ms_u = timed(False)
    xu = d_x.cpu().numpy()
    # end to end through the host call (b in, x out)
    t0 = time.perf_counter()
    xe = B.sirt("sart", ball, K, opts=opts)
    e2e_s = time.perf_counter() - t0
    p1, p2 = B.pass_bytes(True)
    nl = C.c_int64()
    check(lib().fair_batch_launches(B.handle, K, C.byref(nl)))
    per_pass = (nl.value - (0 if args.batch_prec == "f64" else 1)) // (2 * K)
    peak, peak_kind = hbm_peak()
    gbs = (p1 + p2) * K / (ms_b / 1e3) / 1e9
    cpu = None
    if samples:
        snnz = sum(R.nnz for R, _ in samples)
        ro = O.options(lbound=0.0, ubound=1.0)
        t1 = time.perf_counter()
        for R, b in samples:
            O.sirt("sart", R, b, 1, opts=ro)
        ta = time.perf_counter() - t1
        t1 = time.perf_counter()
        for R, b in samples:
            O.sirt("sart", R, b, 3, opts=ro)
        tb = time.perf_counter() - t1
        per_it = max((tb - ta) / 2, 1e-9)  # seconds per iteration of the sample
        cpu = {"value": (snnz / per_it) / info["nnz"], "unit": "batch iter/s", "cores": 1,
               "kind": "port", "sample": f"{len(samples)} of the problems (N <= 160), one SART "
               "iteration (3 minus 1), scaled by nonzeros to the whole batch"}
    line = {"metric": "batched SART iter/s (all problems per iteration)",
            "workload": f"{nprob} fan-beam problems, N 64..512, 90..720 angles, p = ceil(1.42N)",
            "layout": layout, "problem_layouts": shapes,
            "value": K / (ms_b / 1e3), "unit": "batch iter/s", "ms_per_iteration": ms_b / K,
            "iterations": K, "dtype": args.batch_prec, "problems": nprob, "nnz": info["nnz"],
            "device_bytes": info["device_bytes"], "build_s": build_s,
            "unbatched": {"value": K / (ms_u / 1e3), "unit": "batch iter/s",
                          "ms_per_iteration": ms_u / K,
                          "launches_per_iteration": 2 * nprob * (2 if per_pass == 2 else 1),
                          "max_abs_diff_vs_batched": float(np.max(np.abs(xu - xb)))},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": gbs / peak,
                         "algorithmic_bytes_per_iteration": p1 + p2},
            "e2e": {"value": K / e2e_s, "unit": "batch iter/s",
                    "h2d_bytes_per_step": 8 * ball.size / K, "d2h_bytes_per_step": 8 * xe.size / K,
                    "note": "one fair_batch_sirt call of 50 iterations: b uploaded, x downloaded"},
            "gpu_launches": nl.value, "launches_per_pass": per_pass, "pass_config": cfg,
            "clocks": clocks, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)
    B.close()


def run_mfree(args):
    """Matrix-free SIRT (a secondary line): parallel beam N=2048, 1440 angles
    over [0, pi), 2896 bins (7.7e9 nonzeros if stored: 92 GB in FP64 per
    copy), seeded 20-Gaussian phantom, 1% noise, SIRT (Cimmino) 50 iterations
    in FP32 on the matrix-free projector pair (FP64 weights and iterate), and
    on the same matrix stored in FP32 only (A and A' as FP32 values with int64
    row offsets, 123 GB, built by blocks of angles), each arm's iterate
    compared with the other's; beside it, at the N=1024 problem (720 angles,
    1448 bins), the matrix-free and the stored (FP32, autotuned) iterations."""
    import ctypes as C

    import torch

    import fortran_airtools_gb300 as F
    from fortran_airtools_gb300._clib import check, lib
    K = 50
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    out = {}
    sizes = [(2048, 1440, 2896), (1024, 720, 1448)]
    if args.mf_sizes:
        sizes = [s for s in sizes if str(s[0]) in args.mf_sizes.split(",")]
    for n, nth, p in sizes:
        th = np.pi * np.arange(nth) / nth
        d = F.Data(n=n, p=p, nth=nth, theta=th)
        M64 = F.MatrixFree(d, "f64")
        xt = F.phantomgallery.gaussians(n, 20, seed=1)
        b = noisy(M64.project(xt))
        M64.close()
        M = F.MatrixFree(d, "f32")
        nnz = M.nnz()
        M.set_stream(stream.cuda_stream)
        opts = F.airms.options()
        M.prepare("cimmino", opts)
        d_b = torch.from_numpy(b).cuda()
        d_x = torch.zeros(M.n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        M.run_device(d_b.data_ptr(), d_x.data_ptr(), 3)  # warm-up
        stream.synchronize()
        with torch.cuda.stream(stream):
            d_x.zero_()
        sampler = ClockSampler(0)
        sampler.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        M.run_device(d_b.data_ptr(), d_x.data_ptr(), K)
        e1.record(stream)
        stream.synchronize()
        clocks = sampler.stop()
        ms = e0.elapsed_time(e1)
        with torch.cuda.stream(stream):
            d_x.zero_()
        stream.synchronize()
        t1, t2 = M.run_device_timed(d_b.data_ptr(), d_x.data_ptr(), 5)
        res = {"iter_per_s": K / (ms / 1e3), "ms_per_iteration": ms / K,
               "project_ms": t1 / 5, "backproject_ms": t2 / 5, "nnz": nnz,
               "entries_per_s": 2 * nnz / (ms / K / 1e3), "clocks": clocks}
        # the matrix-free iterate after K iterations from zero (error reference)
        with torch.cuda.stream(stream):
            d_x.zero_()
        M.run_device(d_b.data_ptr(), d_x.data_ptr(), K)
        stream.synchronize()
        x_mf = d_x.cpu().numpy()
        M.close()
        if n == 2048 and not args.no_stored:
            res["stored_f32"] = stored_f32_arm(args, F, d, b, x_mf, K, stream, d_b, d_x)
        if n == 1024 and not args.no_stored:  # the stored form, packed FP32, autotuned
            A = F.paralleltomo(d)
            A.set_stream(stream.cuda_stream)
            A.set_precision("f32")
            L = lib()
            check(L.fair_sirt_prepare(A.handle, b"cimmino", C.byref(opts)))
            cfg = (C.c_int32 * 4)()
            check(L.fair_sirt_autotune(A.handle, d_b.data_ptr(), d_x.data_ptr(), 3, cfg))
            with torch.cuda.stream(stream):
                d_x.zero_()
            check(L.fair_sirt_run_device(A.handle, d_b.data_ptr(), d_x.data_ptr(), 3))
            stream.synchronize()
            with torch.cuda.stream(stream):
                d_x.zero_()
            torch.cuda.synchronize()
            e0.record(stream)
            check(L.fair_sirt_run_device(A.handle, d_b.data_ptr(), d_x.data_ptr(), K))
            e1.record(stream)
            stream.synchronize()
            ms_s = e0.elapsed_time(e1)
            res["stored_f32"] = {"iter_per_s": K / (ms_s / 1e3), "ms_per_iteration": ms_s / K,
                                 "pass_config": list(cfg)}
            A.close()
        res["geometry"] = f"parallel beam N={n}, {nth} angles over [0,pi), {p} bins"
        out[f"N={n}"] = res
    if not args.mf_sizes or "fan" in args.mf_sizes.split(","):
        out["fan N=512"] = mfree_fan_case(F, K, stream)
    big = out.get("N=2048") or next(iter(out.values()))
    line = {"metric": "matrix-free SIRT iter/s (Cimmino, FP32)",
            "workload": big["geometry"],
            "value": big["iter_per_s"], "unit": "iter/s", "iterations": K, "dtype": "f32",
            "ms_per_iteration": big["ms_per_iteration"], "nnz_if_stored": big["nnz"],
            "stored_fp64_bytes_per_copy": big["nnz"] * 12,
            "cases": out,
            "note": "matrix-free: nothing of size nnz in memory; the stored form of the N=2048 "
                    "problem needs the FP64 matrix and its transpose while it is built",
            "gpu_launches": 1 + 2 * K}
    print(json.dumps(line), flush=True)
    return 0


def mfree_fan_case(F, K, stream):
    """The fan-beam pair on the Kaczmarz workload's geometry (fan N=512, 720
    angles over [0, 2pi), 725 bins, R = 2N): K FP32 Cimmino iterations on the
    matrix-free pair and on the stored matrix (FP32, autotuned), the iterates
    compared with each other."""
    import ctypes as C

    import torch

    from fortran_airtools_gb300._clib import check, lib
    n, nth, p = 512, 720, 725
    th = 2 * np.pi * np.arange(nth) / nth
    d = F.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th)
    M = F.MatrixFree(d, "f32", beam="fan")
    b = noisy(M.project(F.phantomgallery.shepplogan(n)))
    M.set_stream(stream.cuda_stream)
    opts = F.airms.options()
    M.prepare("cimmino", opts)
    d_b = torch.from_numpy(b).cuda()
    d_x = torch.zeros(M.n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    M.run_device(d_b.data_ptr(), d_x.data_ptr(), 3)  # warm-up
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(run):
        with torch.cuda.stream(stream):
            d_x.zero_()
        torch.cuda.synchronize()
        e0.record(stream)
        run(K)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1), d_x.cpu().numpy()

    ms_mf, x_mf = timed(lambda k: M.run_device(d_b.data_ptr(), d_x.data_ptr(), k))
    with torch.cuda.stream(stream):
        d_x.zero_()
    stream.synchronize()
    t1, t2 = M.run_device_timed(d_b.data_ptr(), d_x.data_ptr(), 3)
    nnz = M.nnz()
    M.close()
    A = F.fanlineartomo(d)
    A.set_stream(stream.cuda_stream)
    A.set_precision("f32")
    L = lib()
    check(L.fair_sirt_prepare(A.handle, b"cimmino", C.byref(opts)))
    cfg = (C.c_int32 * 4)()
    check(L.fair_sirt_autotune(A.handle, d_b.data_ptr(), d_x.data_ptr(), 3, cfg))
    ms_st, x_st = timed(lambda k: check(L.fair_sirt_run_device(A.handle, d_b.data_ptr(),
                                                                 d_x.data_ptr(), k)))
    A.close()
    return {"geometry": f"fan beam N={n}, {nth} angles over [0,2pi), {p} bins, R=2N",
            "iter_per_s": K / (ms_mf / 1e3), "ms_per_iteration": ms_mf / K,
            "project_ms": t1 / 3, "backproject_ms": t2 / 3, "nnz": nnz,
            "stored_f32": {"iter_per_s": K / (ms_st / 1e3), "ms_per_iteration": ms_st / K,
                           "pass_config": list(cfg)},
            "rel_err_vs_stored": float(np.linalg.norm(x_mf - x_st) / np.linalg.norm(x_st))}


def stored_f32_arm(args, F, d, b, x_mf, K, stream, d_b, d_x):
    """The stored-CSR arm of the matrix-free comparison: the same geometry held
    in FP32 only (fair_paralleltomo_f32: A and A' as FP32 values, int32
    columns, int64 row offsets, built by blocks of angles), K Cimmino
    iterations on the CSR layout, timed like the matrix-free ones; the two
    iterates are compared with each other."""
    import ctypes as C

    import torch

    from fortran_airtools_gb300._clib import check, lib
    L = lib()
    t0 = time.perf_counter()
    H = F.paralleltomo_f32(d)
    build_s = time.perf_counter() - t0
    m, n, nnz = H.info()
    H.set_stream(stream.cuda_stream)
    opts = F.airms.options()
    check(L.fair_sirt_prepare(H.handle, b"cimmino", C.byref(opts)))
    out = {"build_s": build_s, "nnz": nnz, "row_offsets": "int64",
           "device_bytes_matrix": int(nnz * 16 + (m + n + 2) * 8)}
    for cfg in ((8, 8, 0, 0), (8, 8, 9, 9)):
        # the CSR, then the tiled copies built beside it (another ~100 GB: if the
        # GPU cannot hold them the line says so)
        st = L.fair_sirt_set_lanes(H.handle, (C.c_int32 * 4)(*cfg))
        if st == 0:
            with torch.cuda.stream(stream):
                d_x.zero_()
            st = L.fair_sirt_run_device(H.handle, d_b.data_ptr(), d_x.data_ptr(), 1)
            stream.synchronize()
        if st != 0:
            out[f"layout_{cfg[2]}_{cfg[3]}"] = {"unavailable": F.FairError(st).args[0]}
            break
        with torch.cuda.stream(stream):
            d_x.zero_()
        check(L.fair_sirt_run_device(H.handle, d_b.data_ptr(), d_x.data_ptr(), 3))  # warm-up
        stream.synchronize()
        with torch.cuda.stream(stream):
            d_x.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        check(L.fair_sirt_run_device(H.handle, d_b.data_ptr(), d_x.data_ptr(), K))
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1)
        x_st = d_x.cpu().numpy()
        ms1, ms2 = C.c_float(), C.c_float()
        with torch.cuda.stream(stream):
            d_x.zero_()
        check(L.fair_sirt_run_device_timed(H.handle, d_b.data_ptr(), d_x.data_ptr(), 3,
                                           C.byref(ms1), C.byref(ms2)))
        gb = 2 * nnz * 8 / 1e9
        key = "csr" if cfg[2] == 0 else f"layout_{cfg[2]}_{cfg[3]}"
        out[key] = {
            "iter_per_s": K / (ms / 1e3), "ms_per_iteration": ms / K,
            "pass1_ms": ms1.value / 3, "pass2_ms": ms2.value / 3,
            "matrix_gbs": gb / (ms / K / 1e3), "pass_config": list(cfg),
            "rel_err_vs_matrix_free": float(np.linalg.norm(x_st - x_mf) / np.linalg.norm(x_mf))}
        if cfg[2] == 9:  # whether the tiled copies were built (else the passes read the CSR)
            out[key]["tiled_built"] = [H.tiled_info()["has"], H.tiled_info(transposed=True)["has"]]
    H.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--prec", choices=["f64", "f32", "f16", "q16"], default="f64")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep 8 lanes per row instead of autotuning each pass")
    ap.add_argument("--lanes", default="",
                    help="fixed lanes per row of pass 1 and pass 2 and optionally groups per lane, "
                         "e.g. 8,4 or 8,4,2,2 (no autotuning)")
    ap.add_argument("--forms", default="f32,f16,q16",
                    help="reduced forms timed after FP64 (comma list of f32, f16, q16)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-oracle baseline")
    ap.add_argument("--no-oracle", action="store_true",
                    help="skip the oracle check (its matrix and iterate) and the CPU baseline")
    ap.add_argument("--n", type=int, default=1024, help="image size N (profiling cases)")
    ap.add_argument("--angles", type=int, default=720)
    ap.add_argument("--bins", type=int, default=1448)
    ap.add_argument("--workload", choices=["sirt", "c1", "kaczmarz", "adjoint", "batch", "mfree"],
                    default="sirt",
                    help="sirt: the headline line; c1, kaczmarz, adjoint, batch, mfree: secondary lines")
    ap.add_argument("--batch-problems", type=int, default=256)
    ap.add_argument("--batch-prec", choices=["f64", "f32", "f16", "q16"], default="f32")
    ap.add_argument("--batch-layout", default="auto,tiled,packed",
                    help="batch layouts timed, one line each (comma list of auto, tiled, packed)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="headline only: skip the secondary workloads run after it")
    ap.add_argument("--kacz-cases", default="",
                    help="kaczmarz workload: cases to run (comma list of randkaczmarz, "
                         "symkaczmarz, kaczmarz; default all)")
    ap.add_argument("--no-stored", action="store_true",
                    help="mfree workload: skip the stored FP32 arms (N=2048 and N=1024)")
    ap.add_argument("--mf-sizes", default="",
                    help="matrix-free cases to run (comma list of 2048, 1024, fan; default all)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global N, NTH, P, WORKLOAD
    N, NTH, P = args.n, args.angles, args.bins
    WORKLOAD = (f"parallel-beam N={N}, {NTH} angles over [0,pi), {P} bins; SIRT (Cimmino)")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "c1":
        return run_c1(args)
    if args.workload == "kaczmarz":
        return run_kaczmarz(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "mfree":
        return run_mfree(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
