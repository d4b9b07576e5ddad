"""Build the CPU oracle shared library (test infrastructure).

``python oracle/build_oracle.py`` compiles ``oracle/atm_oracle.cpp`` into
``oracle/_build/liboracle_atm.so`` with g++.  Flags: ``-ffp-contract=off`` so
that float arithmetic rounds after every operation, as the Taichi reference
does under the f32 interpreter used to pin this oracle; no ``-ffast-math``; no
``-march=native`` (the library is rebuilt on each host, x86 or Arm).
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SOURCE = HERE / "atm_oracle.cpp"
OUTPUT = HERE / "_build" / "liboracle_atm.so"


def build(force: bool = False) -> Path:
    OUTPUT.parent.mkdir(parents=True, exist_ok=True)
    if (
        not force
        and OUTPUT.exists()
        and OUTPUT.stat().st_mtime > SOURCE.stat().st_mtime
        and OUTPUT.stat().st_mtime > (ROOT / "include" / "atm_capi.h").stat().st_mtime
    ):
        return OUTPUT
    tmp = OUTPUT.with_suffix(".so.tmp%d" % os.getpid())
    command = [
        os.environ.get("CXX", "g++"),
        "-O3",
        "-std=c++17",
        "-fPIC",
        "-shared",
        "-fopenmp",
        "-ffp-contract=off",
        "-fno-fast-math",
        "-I",
        str(ROOT / "include"),
        "-o",
        str(tmp),
        str(SOURCE),
    ]
    subprocess.run(command, check=True)
    os.replace(tmp, OUTPUT)
    return OUTPUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
