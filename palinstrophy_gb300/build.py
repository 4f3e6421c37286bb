"""Build libpalgpu.so in-tree for sm_103a (nvcc + g++, translation units in parallel).

    python -m palinstrophy_gb300.build [--force]

Objects go to palinstrophy_gb300/_build/, the library to palinstrophy_gb300/libpalgpu.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import time

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpalgpu.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-I" + INCLUDE, "-I" + CSRC] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I" + INCLUDE]

CU_SOURCES = ["pal_inst_f32_a.cu", "pal_inst_f32_e.cu", "pal_inst_f32_f.cu", "pal_inst_f32_b.cu", "pal_inst_f32_c.cu", "pal_inst_f32_d.cu",
              "pal_inst_f64_a.cu", "pal_inst_f64_b.cu", "pal_inst.cu", "pal_api.cu", "pal_noalloc.cu", "pal_measure.cu",
              "pal_ensemble.cu", "pal_ens_fused.cu", "pal_generate.cu"]
CPP_SOURCES = ["pal_pao.cpp"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = True) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "palgpu.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    gxx = shutil.which("g++") or "g++"
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([gxx] + CXX_FLAGS + ["-c", s, "-o", o])
    t0 = time.time()
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append((j, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + out for j, out in failed)
        raise RuntimeError("libpalgpu build failed:\n" + msg)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        subprocess.check_call([nvcc] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    if verbose:
        print(f"libpalgpu.so ready ({len(jobs)} units rebuilt, {time.time() - t0:.1f}s)")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
