"""Build libracer.so in-tree for sm_103a with nvcc (no cmake, no setuptools).

Translation units compile in parallel to objects under _build/ and link into
_build/libracer.so. The simulator and element-wise PPO kernels (sim.cu,
ppo.cu) are built with --fmad=false and IEEE division/sqrt so they repeat the
CPU restatement's binary32 operations exactly; host code everywhere is built
with -ffp-contract=off so host-side tables (beam directions) match too.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = BUILD / "libracer.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", str(CSRC)]
EXACT = ["--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
UNITS = {
    "sim.cu": EXACT,
    "ppo.cu": EXACT,
    "mlp.cu": [],
    "mlp_tc.cu": EXACT,
    "policy.cu": [],
    "policy_tc.cu": [],
    "api.cu": [],
    "noalloc.cu": [],
    "tma.cu": [],
    "gemm.cu": [],
    "surrogate.cu": [],
    "track.cu": ["--fmad=false", "-ftz=false"],
}


def nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _headers():
    return [p for p in CSRC.glob("*.h")] + [p for p in CSRC.glob("*.cuh")] + [HERE.parent / "include" / "racer.h"]


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose=False, force=False):
    BUILD.mkdir(exist_ok=True)
    headers = _headers()
    jobs = []
    for unit, extra in UNITS.items():
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        if force or _stale(obj, [src, *headers, Path(__file__)]):
            cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
            jobs.append((unit, cmd))

    def run(job):
        unit, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg)
    objs = [BUILD / (u + ".o") for u in UNITS]
    if force or jobs or _stale(LIB, objs):
        tmp = BUILD / f"libracer.{os.getpid()}.so"
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
