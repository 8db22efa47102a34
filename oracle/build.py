"""Build recipes for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles the plain-C restatement ``oracle/src/oracle.c``
  into ``oracle/_build/liboracle.so`` (works on any host with gcc + OpenMP).
* ``build_ref()`` compiles the reference's own CPU operator sources, read in
  place from the reference tree (never copied), together with the small type
  shim in ``oracle/shim`` and the wrapper ``oracle/ref/ref_extras.cpp`` into
  ``oracle/_ref/libsfem_ref.so``.  The reference tree comes from the ``root``
  argument or ``$SFEM_REFERENCE_ROOT``; without either (a machine that only runs the
  tests) it raises with what to set.
"""

from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent

ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libsfem_ref.so"
# the reference's Laplacian sources built again in its float32 number configuration
REF_LIB_F32 = HERE / "_ref" / "libsfem_ref_f32.so"
REF_SOURCES_F32 = ["operators/sshex8/sshex8_laplacian.cpp"]

# reference sources on the operator path (read in place)
REF_SOURCES = [
    "operators/hex8/hex8_laplacian.cpp",
    "operators/hex8/hex8_fff.cpp",
    "operators/sshex8/sshex8_laplacian.cpp",
    "operators/sshex8/sshex8_interpolate.cpp",
    "operators/sshex8/sshex8_linear_elasticity.cpp",
    "operators/hex8/hex8_linear_elasticity.cpp",
]
REF_INCLUDES = [
    "base",
    "operators",
    "operators/hex8",
    "operators/sshex8",
    "operators/stencil",
    "operators/tet4",
    "operators/beam2",
    "algebra",
    "algebra/openmp",
    "frontend/ops/generated",
]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "src" / "oracle.c", HERE / "src" / "solve.c"]
    if force or _stale(ORACLE_LIB, srcs):
        ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
        _run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", str(ORACLE_LIB)] + [str(s) for s in srcs] + ["-lm"])
    return ORACLE_LIB


def reference_root(root=None) -> Path:
    """The reference tree to compile from: ``root``, else ``$SFEM_REFERENCE_ROOT``."""
    r = root if root is not None else os.environ.get("SFEM_REFERENCE_ROOT")
    if not r:
        raise RuntimeError("no reference tree given: pass root=... or set SFEM_REFERENCE_ROOT to the sfem checkout")
    path = Path(r)
    if not (path / "operators" / "sshex8" / "sshex8_laplacian.cpp").exists():
        raise RuntimeError(f"{path} is not an sfem tree (operators/sshex8/sshex8_laplacian.cpp missing)")
    return path


def build_ref(force: bool = False, root=None):
    REF_ROOT = reference_root(root)
    srcs = [REF_ROOT / s for s in REF_SOURCES] + [HERE / "ref" / "ref_extras.cpp"]
    if not (force or _stale(REF_LIB, srcs)):
        return REF_LIB
    objdir = HERE / "_ref" / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = ["-I" + str(HERE / "shim")] + ["-I" + str(REF_ROOT / d) for d in REF_INCLUDES]
    flags = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-DNDEBUG", "-w"] + inc

    def compile_one(src: Path):
        obj = objdir / (src.stem + ".o")
        if force or _stale(obj, [src]):
            _run(flags + ["-c", str(src), "-o", str(obj)])
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, srcs))
    _run(["g++", "-shared", "-fopenmp", "-o", str(REF_LIB)] + [str(o) for o in objs])
    return REF_LIB


def build_ref_f32(force: bool = False, root=None):
    """The reference's sshex8 Laplacian sources with real/scalar/accumulator = float
    (shim_f32 first on the include path) into oracle/_ref/libsfem_ref_f32.so."""
    REF_ROOT = reference_root(root)
    srcs = [REF_ROOT / s for s in REF_SOURCES_F32] + [HERE / "ref" / "ref_f32_extras.cpp"]
    if not (force or _stale(REF_LIB_F32, srcs)):
        return REF_LIB_F32
    objdir = HERE / "_ref" / "obj_f32"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = ["-I" + str(HERE / "shim_f32"), "-I" + str(HERE / "shim")] + ["-I" + str(REF_ROOT / d) for d in REF_INCLUDES]
    flags = ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-DNDEBUG", "-w"] + inc
    objs = []
    for src in srcs:
        obj = objdir / (src.stem + ".o")
        _run(flags + ["-c", str(src), "-o", str(obj)])
        objs.append(obj)
    _run(["g++", "-shared", "-fopenmp", "-o", str(REF_LIB_F32)] + [str(o) for o in objs])
    return REF_LIB_F32


if __name__ == "__main__":
    import sys

    root = sys.argv[1] if len(sys.argv) > 1 else None  # else $SFEM_REFERENCE_ROOT
    print(build_oracle(force=True))
    print(build_ref(force=True, root=root))
    print(build_ref_f32(force=True, root=root))
