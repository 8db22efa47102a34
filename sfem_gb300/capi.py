"""ctypes binding of ``libsfem_gb300.so`` (the C ABI declared in ``include/sfem_gb300.h``).

Device memory is held in torch CUDA tensors; only raw pointers cross the ABI.
The library is loaded from the package tree; a missing library is an error
(there is no CPU fallback on the product path).
"""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "lib" / "libsfem_gb300.so"
HEADER = HERE.parent / "include" / "sfem_gb300.h"

SUCCESS = 0
HEX8 = 8
SSHEX8_BASE = 1000
REAL_DEFAULT, FLOAT32, FLOAT64 = 0, 1, 2
FLOAT32_BF16TC = 3  # float vectors, BF16 tensor-core element contraction (elasticity)


def SSHEX8(L: int) -> int:
    return SSHEX8_BASE + int(L)


_lib = None


class SfemError(RuntimeError):
    pass


def declared_symbols() -> list[str]:
    """Names of every function declared in include/sfem_gb300.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", text, flags=re.M)
    return [n for n in names if not n.startswith("SFEM_GB300_")]


def load(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise SfemError(f"sfem_gb300 CUDA library not built: {p} (run __graft_entry__.build())")
    _lib = C.CDLL(str(p))
    _lib.sfem_gb300_last_error.restype = C.c_char_p
    _lib.sfem_gb300_version.restype = C.c_char_p
    _lib.sfem_gb300_sshex8_packed_bytes.restype = C.c_ssize_t
    return _lib


def last_error() -> str:
    return load().sfem_gb300_last_error().decode()


def check(rc: int, what: str = ""):
    if rc != SUCCESS:
        raise SfemError(f"{what} failed: {last_error()}")


def vp(t) -> C.c_void_p:
    """Raw device pointer of a torch tensor (or None -> NULL)."""
    if t is None:
        return C.c_void_p(0)
    return C.c_void_p(t.data_ptr())


def c_void(addr: int) -> C.c_void_p:
    """Raw address as a pointer argument."""
    return C.c_void_p(int(addr))


def i64(v) -> C.c_ssize_t:
    return C.c_ssize_t(int(v))


class DevicePtrArray:
    """Device array of device pointers to the rows of a 2-D CUDA tensor (``T**``)."""

    def __init__(self, rows):
        import torch

        self.rows = rows.contiguous()
        ptrs = [self.rows[i].data_ptr() for i in range(self.rows.shape[0])]
        self.table = torch.tensor(ptrs, dtype=torch.int64, device=self.rows.device)

    @property
    def ptr(self) -> C.c_void_p:
        return C.c_void_p(self.table.data_ptr())

    @property
    def n(self) -> int:
        return self.rows.shape[1]


def real_type_of(t) -> int:
    import torch

    if t.dtype == torch.float64:
        return FLOAT64
    if t.dtype == torch.float32:
        return FLOAT32
    raise SfemError(f"unsupported dtype {t.dtype}")
