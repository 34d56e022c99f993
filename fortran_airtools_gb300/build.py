"""Build the GB300 library libfair_gb300.so in-tree with nvcc.

Every translation unit under csrc/ is compiled for sm_103a only (one
-gencode, no PTX for other targets) in parallel, then linked into
fortran_airtools_gb300/_lib/libfair_gb300.so against the shared CUDA runtime;
the main.exe drop-in (cli/fair_main.cpp) is linked against it as
_lib/fair_main.
Host code is compiled with -ffp-contract=off so that host-side geometry
tables round every product separately (aarch64 g++ would otherwise fuse
multiply-adds).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libfair_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def common_flags():
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _compile(args):
    nvcc, src, obj, extra = args
    cmd = [nvcc, "-c", src, "-o", obj] + common_flags() + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile and link; returns the path of the shared library."""
    nvcc = nvcc_path()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = sources()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    jobs = []
    for s in srcs:
        obj = os.path.join(BUILD_DIR, os.path.basename(s)[:-3] + ".o")
        jobs.append((nvcc, s, obj, extra))
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        results = list(ex.map(_compile, jobs))
    failed = [(s, out) for s, rc, out in results if rc != 0]
    for s, rc, out in results:
        if verbose or rc != 0 or ptxas_info:
            if out.strip():
                print(f"--- {os.path.basename(s)}\n{out}", file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(s) for s, _ in failed))
    lib = os.path.join(OUT_DIR, LIB_NAME)
    cudalib = os.path.join(cuda_home(nvcc), "lib64")
    cmd = [nvcc, "-shared", "-o", lib, ARCH, "-cudart", "shared",
           "-Xlinker", f"-rpath,{cudalib}"] + [j[2] for j in jobs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    build_cli(nvcc)
    return lib


def build_cli(nvcc: str) -> str:
    """The main.exe drop-in, linked against the library beside it."""
    exe = os.path.join(OUT_DIR, "fair_main")
    cmd = [nvcc, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "cli", "fair_main.cpp"),
           "-I", os.path.join(ROOT, "include"), "-L", OUT_DIR, "-lfair_gb300",
           "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("fair_main build failed:\n" + r.stdout + r.stderr)
    return exe


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
