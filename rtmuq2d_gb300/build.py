"""In-tree build of the engine library (librtmgpu.so) for sm_103a.

Plain nvcc / gcc invocations, translation units compiled in parallel, output in
rtmuq2d_gb300/_build/.  Used by __graft_entry__.build() and by the package loader when
the library is missing.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "librtmgpu.so")
DROPIN_LIB = os.path.join(OUT, "librtm_dropin.so")     # the reference's entry-point names

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
              "-I" + CSRC, "--expt-relaxed-constexpr"]
CC_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-std=gnu99", "-I" + INCLUDE]

CU_SOURCES = ["rtm_kernels.cu", "rtm_engine.cu"]
C_SOURCES = ["rtm_host.c", "rtm_zfp.c", "rtm_driver.c"]
DROPIN_SOURCES = ["rtm_dropin.c"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _newer(target: str, sources) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + \
           [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if not force and _newer(LIB, deps) and _newer(DROPIN_LIB, deps):
        return LIB
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + \
              ["-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append((cmd, obj))
    for src in C_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        jobs.append((["gcc"] + CC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj], obj))
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose or ptxas_info:
        for log in logs:
            if log.strip():
                sys.stderr.write(log)
    tmp = LIB + ".tmp"
    _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for _, o in jobs] + ["-lcudart"])
    os.replace(tmp, LIB)
    # the drop-in library: the reference's names over librtmgpu (found next to it)
    objs = []
    for src in DROPIN_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        _run(["gcc"] + CC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    tmp = DROPIN_LIB + ".tmp"
    _run(["gcc", "-shared", "-o", tmp] + objs + ["-L" + OUT, "-lrtmgpu", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, DROPIN_LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="-v" in sys.argv)
    print(LIB)
