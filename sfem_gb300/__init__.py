"""sfem_gb300: GB300-native (sm_103a) matrix-free operator path for sshex8 / hex8 meshes.

The compute path is the CUDA library ``lib/libsfem_gb300.so`` behind the C ABI
in ``include/sfem_gb300.h``; this package holds its ctypes binding
(:mod:`sfem_gb300.capi`), the host-side mirror of the reference's operator
interface (:mod:`sfem_gb300.ops`) and the semi-structured mesh layer
(:mod:`sfem_gb300.mesh`) that stands in for the reference's smesh submodule.
"""

from . import capi, mesh  # noqa: F401

__all__ = ["capi", "mesh"]
