"""The header-only C++ adapter (include/sfem_gb300_adapter.hpp) compiled against the C
ABI: on the CPU the header compiles and links (every adapter instantiated on the
reference-shaped interfaces); on the GPU the compiled test runs the BLAS, Operator and
Op adapters through a CG solve and operator identities (tests/cpp/test_adapter.cpp)."""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CUDA = Path("/usr/local/cuda")


def _build(tmp_path):
    from sfem_gb300 import capi

    lib = capi.LIB_PATH
    if not lib.exists():
        pytest.skip("CUDA library not built")
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "test_adapter"
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "cpp" / "test_adapter.cpp"), "-o", str(exe), "-L", str(lib.parent), "-lsfem_gb300",
           "-L", str(CUDA / "lib64"), "-lcudart", f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_adapter_compiles_and_links(tmp_path):
    _build(tmp_path)


@pytest.mark.gpu
def test_adapter_on_gpu(cuda, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all checks passed" in r.stdout
