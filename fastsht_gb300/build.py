"""Builds the fastsht_gb300 CUDA library in-tree (sm_103a only).

    python -m fastsht_gb300.build          # -> fastsht_gb300/_lib/libfastsht_gb300.so

Translation units compile in parallel with nvcc, then link into one shared
library with a static CUDA runtime, so the .so depends only on the driver.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB_NAME = "libfastsht_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastsht_gb300")


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def sources():
    return sorted(CSRC.glob("*.cu"))


def _needs_rebuild(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    obj_dir = OUT_DIR / "obj"
    obj_dir.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((PKG.parent / "include").glob("*.h"))
    srcs = sources()
    nv = nvcc()

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.stem + ".o")
        if force or _needs_rebuild(obj, [src] + headers):
            cmd = [nv, *ARCH, *NVCC_FLAGS, "-I", str(PKG.parent / "include"), "-c", str(src),
                   "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
            if verbose and r.stderr.strip():
                print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    lib = lib_path()
    if force or _needs_rebuild(lib, objs):
        tmp = lib.with_suffix(".so.tmp")
        cmd = [nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
