"""Build the engine library ``liboafdtd.so`` for sm_103a with nvcc (no torch, no cmake).

``python -m open_analysis_gb300.build`` compiles every ``csrc/*.cu`` translation unit in parallel
and links them into ``open_analysis_gb300/lib/liboafdtd.so`` in the source tree. The library is
built with ``-fmad=false``: the kernels then round every multiply and add separately, exactly as
the NumPy reference does, so float32 fields agree bit for bit with the reference's float32 run.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
LIBNAME = "liboafdtd.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false keeps the device arithmetic unfused; -ffp-contract=off does the same for host code
# (GCC fuses multiply-add by default on Arm), which the native model compiler needs to equal NumPy
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the engine library needs the CUDA toolkit to build")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile and link; returns the library path. Rebuilds only what is out of date."""
    exe = nvcc()
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((PKG.parent / "include").glob("*.h"))
    extra = extra or []
    jobs = []
    for src in sources():
        obj = objdir / (src.stem + ".o")
        if force or _stale(obj, [src, *headers, Path(__file__)]):
            cmd = [exe, *ARCH, *FLAGS, *extra, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd: list[str]) -> None:
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr, flush=True)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as pool:
        list(pool.map(run, jobs))
    objs = [objdir / (s.stem + ".o") for s in sources()]
    out = lib_path()
    if force or jobs or _stale(out, objs):
        run([exe, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart"])
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(lib_path())
