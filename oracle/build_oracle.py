"""Compiles the oracle's C restatement (oracle/plm.c) into oracle/_build/.

Test infrastructure: only tests/, __graft_entry__ and bench.py's CPU-baseline leg
use it.  Plain gcc, no -march flags (the same source builds on x86_64 and aarch64).
"""
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle_plm.so"


def build(force: bool = False) -> Path:
    src = HERE / "plm.c"
    if not force and OUT.exists() and OUT.stat().st_mtime >= src.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-fopenmp", "-shared", "-fPIC", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
