"""Host-side mirror of the reference's operator interface on the GPU path.

The reference's ``sfem::Op`` (``frontend/ops/sfem_Op.hpp:42-324``) exposes
``initialize``, ``apply(x, h, out)`` (out += H h), ``hessian_diag`` and
``derefine_op``; its GPU ops (``frontend/cuda/sfem_Function_incore_cuda.cpp``:
``GPULaplacian`` 545-751, ``GPULinearElasticity`` 753-1013) cache device
geometry (FFF SoA float, adjugate SoA float) in ``initialize`` and call the C
ABI.  The classes here do the same on top of ``libsfem_gb300.so``: device
buffers are torch CUDA tensors, every call goes through the C ABI.

``SSMeshDevice`` uploads one level of an :class:`sfem_gb300.mesh.SSMesh`
(connectivity, points, Dirichlet nodes) -- the role of the reference's
``FunctionSpace`` device elements.
"""

from __future__ import annotations

import numpy as np

from . import capi
from .mesh import SSMesh


class SSMeshDevice:
    """One level ``l`` of a semi-structured mesh hierarchy, resident on the GPU."""

    def __init__(self, mesh: SSMesh, level: int | None = None, device="cuda:0"):
        import torch

        self.mesh = mesh
        self.level = mesh.L if level is None else int(level)
        self.device = torch.device(device)
        self.n_elements = mesh.n_elements
        self.n_nodes = mesh.n_nodes(self.level)
        if self.level == 1:
            el = mesh.hex8_elements()
            self.element_type = capi.HEX8
        else:
            el = mesh.elements(self.level)
            self.element_type = capi.SSHEX8(self.level)
        self.elements_host = el
        self.elements = torch.from_numpy(np.ascontiguousarray(el)).to(self.device)
        self.elements_ptrs = capi.DevicePtrArray(self.elements)
        # macro corners (hex8 order) for geometry
        if self.level == 1:
            corners = el
        else:
            corners = el[mesh.macro_corner_lidx(self.level)]
        self.corners = torch.from_numpy(np.ascontiguousarray(corners)).to(self.device)
        self.corners_ptrs = capi.DevicePtrArray(self.corners)
        self.points = torch.from_numpy(np.ascontiguousarray(mesh.points)).to(self.device)
        self.points_ptrs = capi.DevicePtrArray(self.points)

    def dirichlet_nodes(self, faces=("x0",)):
        import torch

        ids = np.unique(np.concatenate([self.mesh.boundary_nodes(f, self.level) for f in faces])).astype(np.int32)
        return torch.from_numpy(ids).to(self.device)


class Laplacian:
    """Matrix-free Laplacian op on the GPU (mirror of ``GPULaplacian``)."""

    def __init__(self, space: SSMeshDevice, coefficient=None, packed=True):
        self.space = space
        self.coefficient = coefficient
        self.fff = None
        # applies of sshex8 L = 4 read the connectivity + metric repacked into one
        # contiguous block per 32 macro elements (built with the metric)
        self.packed = bool(packed)
        self.packed_blocks = None

    def initialize(self, stream=None):
        import torch

        E = self.space.n_elements
        self.fff = torch.empty((6, E), dtype=torch.float32, device=self.space.device)
        capi.check(
            capi.load().sfem_gb300_hex8_fff_fill(capi.i64(E), self.space.corners_ptrs.ptr, self.space.points_ptrs.ptr,
                                                 capi.i64(E), capi.vp(self.fff), None),
            "sfem_gb300_hex8_fff_fill")
        if self.coefficient is not None:
            # per-macro-element coefficient k_e scales the metric exactly
            k = torch.as_tensor(self.coefficient, dtype=torch.float32, device=self.space.device)
            self.fff *= k[None, :]
        return self._pack()

    def _pack(self):
        import torch

        self.packed_blocks = None
        lib = capi.load()
        E = self.space.n_elements
        nbytes = lib.sfem_gb300_sshex8_packed_bytes(self.space.element_type, capi.i64(E)) if self.packed else -1
        if nbytes > 0:
            self.packed_blocks = torch.empty(nbytes // 4, dtype=torch.int32, device=self.space.device)
            capi.check(lib.sfem_gb300_sshex8_pack(self.space.element_type, capi.i64(E), self.space.elements_ptrs.ptr,
                                                  capi.i64(self.fff.shape[1]), capi.vp(self.fff),
                                                  capi.vp(self.packed_blocks), None),
                       "sfem_gb300_sshex8_pack")
        return self

    def set_fff(self, fff_soa):
        """Use an externally computed SoA float32 FFF ``[6, E]``."""
        import torch

        self.fff = torch.as_tensor(fff_soa, dtype=torch.float32, device=self.space.device).contiguous()
        return self._pack()

    def apply(self, x, out, stream=None):
        """out += A x (x, out: float32 or float64 CUDA tensors)."""
        E = self.space.n_elements
        rt = capi.real_type_of(x)
        if self.packed_blocks is not None and rt in (capi.FLOAT32, capi.FLOAT64):
            capi.check(
                capi.load().sfem_gb300_sshex8_laplacian_apply_packed(self.space.element_type, capi.i64(E),
                                                                     capi.vp(self.packed_blocks), rt, capi.vp(x),
                                                                     capi.vp(out), stream),
                "sfem_gb300_sshex8_laplacian_apply_packed")
            return out
        capi.check(
            capi.load().cu_laplacian_apply(self.space.element_type, capi.i64(E), self.space.elements_ptrs.ptr,
                                           capi.i64(E), capi.vp(self.fff), capi.real_type_of(x), capi.vp(x),
                                           capi.vp(out), stream),
            "cu_laplacian_apply")
        return out

    def hessian_diag(self, out, stream=None):
        E = self.space.n_elements
        capi.check(
            capi.load().cu_laplacian_diag(self.space.element_type, capi.i64(E), self.space.elements_ptrs.ptr,
                                          capi.i64(E), capi.vp(self.fff), capi.real_type_of(out), capi.vp(out), stream),
            "cu_laplacian_diag")
        return out
