"""Build recipe of the oracle's C restatement (test infrastructure).

Compiles ``oracle/ints_ref.c`` with gcc into ``oracle/_build/libints_ref.so``
(OpenMP across the host cores).  Called by ``__graft_entry__.build()``; the
product never loads the result.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libints_ref.so"
SRC = HERE / "ints_ref.c"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("gcc is required to build the oracle's C restatement")
    OUT.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed on {SRC.name}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
