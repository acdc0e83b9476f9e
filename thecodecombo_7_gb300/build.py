"""Builds libfe.so (the force engine) with nvcc for sm_103a.

Each .cu is compiled separately and in parallel; the FP64 drop-in units get
-fmad=false so that every multiply and add rounds separately as in the
reference's C (bit-exact neighbour-list pair sets, forces equal to the
reference's up to the order of the final sums).  The mixed-precision units
keep FMA contraction.

    python -m thecodecombo_7_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfe.so")
HOSTLIB = os.path.join(HERE, "libfe_sysgen.so")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
# translation unit -> extra flags
UNITS = {
    "fe_api.cu": ["-Xcompiler", "-ffp-contract=off"],
    "k_nblist.cu": ["-fmad=false"],
    "k_pair64.cu": ["-fmad=false"],
    "k_bonded_ext.cu": ["-fmad=false"],
    "k_spme.cu": ["-fmad=false"],
    "k_integrate.cu": ["-fmad=false"],
    "k_integrate_mx.cu": [],
    "k_respa.cu": ["-fmad=false"],
    "k_mc.cu": ["-fmad=false"],
    "k_mixed.cu": ["-ftz=true"],
    "k_noalloc.cu": [],
    "k_replica.cu": ["-fmad=false"],
    "k_mcrun.cu": ["-ftz=true"],
    "k_mlp.cu": [],
    "k_go.cu": [],
    "k_peaks.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the force engine needs the CUDA toolkit to build")


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + [
        os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _compile(src: str, obj: str, extra) -> str:
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_host(force: bool = False) -> str:
    """The workload generator's host helper (plain C, gcc)."""
    src = os.path.join(CSRC, "sysgen.c")
    if force or not os.path.exists(HOSTLIB) or os.path.getmtime(HOSTLIB) < os.path.getmtime(src):
        tmp = HOSTLIB + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared",
                               "-ffp-contract=off", "-o", tmp, src, "-lm"])
        os.replace(tmp, HOSTLIB)
    return HOSTLIB


def build(force: bool = False, verbose: bool = False) -> str:
    build_host(force)
    os.makedirs(BUILD, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    hdr_time = max(os.path.getmtime(h) for h in _headers())
    jobs = []
    objs = []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(
                os.path.getmtime(src), hdr_time):
            jobs.append((src, obj, UNITS[u]))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for obj in ex.map(lambda j: _compile(*j), jobs):
                if verbose:
                    print("compiled", os.path.basename(obj))
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcufft", "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
