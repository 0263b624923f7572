"""Build the sm_103a shared library ``libgomc_gb300.so`` in-tree.

Each CUDA translation unit under ``gomc_gb300/csrc`` is compiled by nvcc in
parallel for ``compute_103a/sm_103a`` and linked into
``gomc_gb300/_build/libgomc_gb300.so`` (the C ABI of include/gomc_gb300.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgomc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is built without floating-point contraction so that x86-64 and
# aarch64 hosts round the set-up arithmetic (k-vectors, prefactors) the same
# way the reference's host build does.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
              "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu"))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "gomc_gb300.h"))
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + (extra or []) + [
                "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd),
                                                        p.stderr[-6000:]))
        if verbose and p.stderr:
            sys.stderr.write(p.stderr)
        return cmd

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".%d.tmp" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n%s" % p.stderr[-4000:])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
