"""Build recipe for the sfem_gb300 CUDA library (sm_103a only).

Compiles every ``csrc/*.cu`` (and ``csrc/*.cpp``) translation unit with nvcc
for ``-gencode arch=compute_103a,code=sm_103a`` in parallel and links
``sfem_gb300/lib/libsfem_gb300.so``.  No cmake, no torch extension machinery.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
LIB = HERE / "lib" / "libsfem_gb300.so"
OBJ = HERE / "lib" / "obj"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list((ROOT / "include").glob("*.h")))


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _flags(extra=()):
    return [
        nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
        "-I" + str(ROOT / "include"), "-I" + str(CSRC), *extra,
    ]


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    srcs = _sources()
    hdrs = _headers()
    OBJ.mkdir(parents=True, exist_ok=True)

    def compile_one(src: Path) -> Path:
        obj = OBJ / (src.name + ".o")
        if force or _stale(obj, [src, *hdrs]):
            cmd = _flags(extra_flags) + ["-c", str(src), "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 2))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True))
