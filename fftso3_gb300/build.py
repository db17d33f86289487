"""Builds the CUDA library ``libfftso3_gb300.so`` for sm_103a (GB300).

Every translation unit under ``csrc/`` is compiled by nvcc in parallel into
``_build/`` and linked into one shared library next to this file.  The
Wigner-d / Legendre table unit is compiled with ``-fmad=false`` so that the
reference-faithful recursions keep the reference's rounding (no fused
multiply-add contraction).
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
LIB = os.path.join(HERE, "libfftso3_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr",
          "-I", os.path.join(HERE, "..", "include")]
PER_FILE = {"tables.cu": ["-fmad=false"], "noalloc.cu": ["-fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "fftso3_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    jobs = []
    for f in sources():
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f.replace(".cu", ".o"))
        if _stale(obj, src):
            cmd = [cc, *ARCH, *COMMON, *PER_FILE.get(f, []), *(extra or []), "-c", src, "-o", obj]
            jobs.append((f, cmd))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): f for f, cmd in jobs}
            errs = []
            for fut in cf.as_completed(futs):
                r = fut.result()
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout, r.stderr, file=sys.stderr)
                if r.returncode != 0:
                    errs.append(f"{futs[fut]}:\n{r.stderr}")
            if errs:
                raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [os.path.join(BUILD, f.replace(".cu", ".o")) for f in sources()]
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
