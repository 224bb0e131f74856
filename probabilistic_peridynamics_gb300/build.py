"""Build the CUDA C-ABI library ``libpp_gb300.so`` in-tree.

Compiles every ``csrc/*.cu`` for sm_103a in parallel (one ``nvcc`` per
translation unit) and links them into ``libpp_gb300.so`` next to this file.
Objects go to ``_build/``.  A unit is recompiled only when it or a header is
newer than its object.

Usage: ``python -m probabilistic_peridynamics_gb300.build [--force]``.
"""
import concurrent.futures
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE.parent / "_build" / "pp_gb300"
LIB = HERE / "libpp_gb300.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE)]
#: Per-unit flags.  The mixed-precision step accepts flushed denormals and
#: approximate FP32 division/square root: its error band covers them.
_FAST_FP32 = ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
UNIT_FLAGS = {"pp_mixed": _FAST_FP32, "pp_tiled": _FAST_FP32}


def _nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = pathlib.Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build")


def _headers():
    return list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale(src, obj, headers):
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *headers])


def build(force=False, verbose=False):
    """Compile and link; returns the path of the shared library."""
    nvcc = _nvcc()
    BUILD.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = _headers()
    objects = [BUILD / (s.stem + ".o") for s in sources]
    jobs = [(s, o) for s, o in zip(sources, objects)
            if force or _stale(s, o, headers)]

    def compile_one(job):
        src, obj = job
        extra = [f for prefix, flags in UNIT_FLAGS.items()
                 if src.name.startswith(prefix) for f in flags]
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o",
               str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stderr}")
        return obj

    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(workers) as pool:
            list(pool.map(compile_one, jobs))
    if force or jobs or not LIB.exists() or any(
            o.stat().st_mtime > LIB.stat().st_mtime for o in objects):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp),
               *[str(o) for o in objects], "-cudart", "static"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
