"""Build libplanet_atm.so (the C ABI of include/atm_capi.h) for sm_103a.

    python planet-real-time-render_gb300/build_native.py [--force] [--jobs N]

Compiles every ``csrc/*.cu`` translation unit in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and links them
into ``planet_renderer_gb300/lib/libplanet_atm.so`` (in-tree, git-ignored).
Only symbols declared ``extern "C"`` with default visibility are exported.
Object files are reused when newer than their sources and headers.
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
INCLUDE = ROOT / "include"
OBJ_DIR = HERE / "_build"
LIB_DIR = HERE / "planet_renderer_gb300" / "lib"
LIBRARY = LIB_DIR / "libplanet_atm.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "-Xptxas",
    "-v",
]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    default = Path("/usr/local/cuda/bin/nvcc")
    if default.exists():
        return str(default)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libplanet_atm")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(source: Path, force: bool) -> tuple[Path, str]:
    obj = OBJ_DIR / (source.stem + ".o")
    if not force and not _stale(obj, [source] + _headers()):
        return obj, ""
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(source), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {source.name}:\n{proc.stdout}\n{proc.stderr}")
    return obj, proc.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    jobs = jobs or min(len(sources), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as pool:
        results = list(pool.map(lambda s: _compile(s, force), sources))
    objects = [obj for obj, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log, file=sys.stderr)
    if force or _stale(LIBRARY, objects):
        tmp = LIBRARY.with_suffix(".so.tmp%d" % os.getpid())
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objects)]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{proc.stdout}\n{proc.stderr}")
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    parser = argparse.ArgumentParser()
    parser.add_argument("--force", action="store_true")
    parser.add_argument("--jobs", type=int)
    parser.add_argument("--verbose", action="store_true")
    args = parser.parse_args()
    print(build(force=args.force, jobs=args.jobs, verbose=args.verbose))
