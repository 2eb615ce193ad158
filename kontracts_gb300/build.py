"""Build the engine's shared library in-tree: kontracts_gb300/libkontract_gpu.so.

Host C++ (frontend, C ABI) is compiled with g++, device code with nvcc for
sm_103a only; translation units are compiled in parallel and linked with
nvcc. Objects go to kontracts_gb300/_build/.

    python -m kontracts_gb300.build            # build if sources changed
    python -m kontracts_gb300.build --force    # rebuild everything
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libkontract_gpu.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXX_SOURCES = ["frontend.cpp", "capi.cpp"]
CU_SOURCES = ["engine.cu", "paths_gbm.cu", "paths_heston.cu", "batch.cu", "lsm.cu", "adjoint.cu",
              "fixed_scratch.cu", "book.cu", "paths_pair.cu", "paths_multi.cu",
              "paths_multi_lean.cu", "paths_mlmc.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "kontract_gpu.h"))
    return hs


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + _headers())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for f in CXX_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I", INCLUDE, "-c", src, "-o", obj])
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            # host code rounds every product and sum (no a * b + c contraction, as the
            # reference's Rust and the oracle): step tables and closed forms agree bit for bit
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "--expt-relaxed-constexpr", "-I", INCLUDE, "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if out and (verbose or p.returncode or ptxas_info):
            sys.stdout.write(out)
        if p.returncode:
            failed.append(cmd[-3])
    if failed:
        raise RuntimeError(f"compilation failed: {failed}")
    if jobs or force or not os.path.exists(LIB):
        link = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        if verbose:
            print(" ".join(link), flush=True)
        subprocess.run(link, check=True)
    return LIB


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose, ptxas_info=a.ptxas_info))


if __name__ == "__main__":
    main()
