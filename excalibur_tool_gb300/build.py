"""Build recipe for libexcalibur_gb300.so (sm_103a), in-tree, without cmake.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library next to this file. The parity units (exc_exact_*.cu) are compiled
with --fmad=false so no multiply-add is contracted. The *_slow units hold the
tracer kernels of launches with a slow-Interpolator field.
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
LIB = os.path.join(HERE, "libexcalibur_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
UNITS = {
    **{f"exc_exact_{s}.cu": ["--fmad=false"] for s in ("rk4", "rk45", "lf4", "aux")},
    **{f"exc_fast_{s}.cu": ["--fmad=true"] for s in ("rk4", "rk45", "lf4", "aux")},
    **{f"exc_exact_{s}_slow.cu": ["--fmad=false"] for s in ("rk4", "rk45", "lf4")},
    **{f"exc_fast_{s}_slow.cu": ["--fmad=true"] for s in ("rk4", "rk45", "lf4")},
    "exc_mixed.cu": ["--fmad=true"],
    "exc_capi.cu": [],
    "exc_noalloc.cu": [],
    "exc_mlp.cu": [],
    "exc_tune.cu": [],
    "exc_gen.cu": ["--fmad=false"],
    "exc_born.cu": [],
    "exc_probe.cu": ["--fmad=false"],
    "exc_maps.cu": ["--fmad=false"],
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".inc"))]
    headers.append(os.path.join(HERE, "..", "include", "excalibur_gb300.h"))
    jobs = []
    objs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
        stamp = obj + ".cmd"      # the command that built the object: a change of flags rebuilds it
        same_cmd = os.path.exists(stamp) and open(stamp).read() == " ".join(cmd)
        if force or not same_cmd or _sources_newer(obj, [src] + headers):
            jobs.append((unit, cmd))

    def run(job):
        unit, cmd = job
        p = subprocess.run(cmd, capture_output=True, text=True)
        return unit, cmd, p

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for unit, cmd, p in ex.map(run, jobs):
            log = os.path.join(BUILD, unit + ".log")
            with open(log, "w") as fh:
                fh.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
            if p.returncode != 0:
                sys.stderr.write(p.stdout + p.stderr)
                raise RuntimeError(f"nvcc failed for {unit} (see {log})")
            with open(os.path.join(BUILD, unit.replace(".cu", ".o")) + ".cmd", "w") as fh:
                fh.write(" ".join(cmd))
            if verbose:
                sys.stderr.write(f"[build] {unit} ok\n")
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "shared",
               "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            sys.stderr.write(p.stdout + p.stderr)
            raise RuntimeError("link of libexcalibur_gb300.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
