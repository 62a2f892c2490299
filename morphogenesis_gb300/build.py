"""Build recipe of the GB300 extension: nvcc, sm_103a only, in-tree output.

The shared library ``_build/libmg_gb300.so`` exports the C-ABI declared in
``include/mg_abi.h``.  Physics translation units are compiled with ``-fmad=false`` so the
kernels evaluate the reference kernels' float expressions without fused multiply-adds.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
# MG_BUILD_DIR (environment, a directory name inside the package) builds a variant elsewhere,
# e.g. the bounds-checking library (MG_NVCC_EXTRA=-DMG_BOUNDS_CHECK=1) next to the product one
OUT = PKG / os.environ.get("MG_BUILD_DIR", "_build")
LIB = OUT / "libmg_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]
# translation unit -> extra flags
UNITS = {
    "mg_sort.cu": ["-fmad=false"],
    "mg_physics.cu": ["-fmad=false"],
    "mg_io.cu": [],
    "mg_mlp.cu": [],
    "mg_api.cu": [],
    "mg_noalloc.cu": [],
    "mg_remodel.cu": ["-fmad=false"],
    "mg_files.cpp": [],
}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA extension cannot be built")
    return exe


def _sources_newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles what changed.  MG_NVCC_EXTRA (environment) adds flags to every unit, e.g.
    -DMG_NL_CAP=64 -DMG_DENS_WARPS=6 to try another density-pass configuration."""
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "mg_abi.h"]
    user = os.environ.get("MG_NVCC_EXTRA", "").split()
    stamp = OUT / "flags.txt"
    if not stamp.exists() or stamp.read_text() != " ".join(user):
        force = True
    objs = []
    jobs = []
    for unit, extra in UNITS.items():
        src = CSRC / unit
        obj = OUT / (unit + ".o")
        objs.append(obj)
        if force or _sources_newer(obj, [src, *headers, Path(__file__)]):
            cmd = [nvcc(), *ARCH, *COMMON, *extra, *user, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _sources_newer(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        run(cmd)
    stamp.write_text(" ".join(user))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
