"""Differentiable signed distance field of a triangle mesh (PyTorch).

``sdf(vertices, plan)`` returns the signed distance of every cell of the plan's
grid to the mesh (negative inside, sign from the exact-predicate occupancy) as an
``(nx, ny, nz)`` tensor, the array layout of the reference binding's
``voxelize`` (bindings/python/src/cybermesh/__init__.py:439-495). Its backward
is the hand-written adjoint of libcmg_c.so: only the per-cell nearest triangle
and Ericson region (src/voxelize/voxelize.cpp:202-247) are kept from the
forward, the closest points are recomputed in FP64, and the per-vertex sums run
in a fixed order, so gradients are bitwise reproducible.

    plan = SDFPlan(vertices, faces, grid=(corner, spacing, (nx, ny, nz)))
    v = torch.tensor(vertices, device="cuda", requires_grad=True)
    loss = ((sdf(v, plan) - target) ** 2).sum()
    loss.backward()            # v.grad: dL/dv

PyTorch is used for device memory and streams only; the work runs in the
library's CUDA kernels (there is no CPU path).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import PREC_FP64, PRED_COMPAT, _check, _clib, make_opts
from . import _lib as _L


def _err():
    return ctypes.create_string_buffer(512)


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class SDFPlan:
    """One mesh of fixed topology on an explicit grid: forwards at moving vertex
    positions and their adjoints (``cmg_sdf_plan_*`` in cmg_gpu.h).

    ``grid`` is ``(corner, spacing, dims)``: the min corner of cell (0, 0, 0), the
    cubic cell edge and ``(nx, ny, nz)``. ``precision`` is ``PREC_FP64`` (plain,
    bit-identical to the reference's distances) or ``PREC_MIXED``. ``autotune`` times
    the pipeline's tunables on this mesh and grid at creation (brick edge, queue grab,
    walk warps, probe head, evaluation CTAs per SM) and keeps the fastest; ``tuning``
    (keys of ``make_opts``) sets them instead."""

    def __init__(self, vertices, faces, grid, precision: int = PREC_FP64,
                 predicates: int = PRED_COMPAT, band: float = 1.0, brick: int = 0,
                 autotune: bool = False, **tuning):
        v = np.ascontiguousarray(
            vertices.detach().cpu().numpy() if isinstance(vertices, torch.Tensor) else vertices,
            dtype=np.float64)
        f = np.ascontiguousarray(
            faces.detach().cpu().numpy() if isinstance(faces, torch.Tensor) else faces,
            dtype=np.int32)
        if v.ndim != 2 or v.shape[1] != 3 or f.ndim != 2 or f.shape[1] != 3:
            raise ValueError("vertices must be (V, 3) and faces (T, 3)")
        corner, spacing, dims = grid
        self.dims = tuple(int(d) for d in dims)
        self.corner = tuple(float(c) for c in corner)
        self.spacing = float(spacing)
        self.npoints, self.ntriangles = len(v), len(f)
        o = make_opts(outputs=0, precision=precision, predicates=predicates, grid=grid,
                      band=band, brick=brick, autotune=autotune, **tuning)
        out = ctypes.c_void_p()
        err = _err()
        _check(_clib.cmg_sdf_plan_create(v.ctypes.data_as(_L.c_double_p), len(v),
                                         f.ctypes.data_as(_L.c_int_p), len(f), ctypes.byref(o),
                                         ctypes.byref(out), err, 512), err)
        self._h = out.value
        self.cells = int(_clib.cmg_sdf_plan_cells(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            _clib.cmg_sdf_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _points(self, vertices: torch.Tensor) -> torch.Tensor:
        if not vertices.is_cuda:
            raise ValueError("vertices must be a CUDA tensor")
        if tuple(vertices.shape) != (self.npoints, 3):
            raise ValueError(f"vertices must have shape ({self.npoints}, 3)")
        return vertices.detach().to(torch.float64).contiguous()

    def forward(self, vertices: Optional[torch.Tensor]) -> Tuple[torch.Tensor, ...]:
        """(sdf float64, occupancy uint8, nearest triangle int32, region uint8), each
        a flat tensor of the grid's cells (idx = (k*ny + j)*nx + i). ``vertices=None``
        reuses the last positions (no re-sizing, nothing synchronised)."""
        if vertices is None:
            if getattr(self, "_device", None) is None:
                raise ValueError("the first forward needs vertices")
            p, dev, ptr = None, self._device, 0
        else:
            p = self._points(vertices)
            dev, ptr = p.device, p.data_ptr()
            self._device = dev
        err = _err()
        with torch.cuda.device(dev):
            st = _stream()
            _check(_clib.cmg_sdf_plan_forward(self._h, ptr, st, err, 512), err)
            n = self.cells
            sdf = torch.empty(n, dtype=torch.float64, device=dev)
            occ = torch.empty(n, dtype=torch.uint8, device=dev)
            tri = torch.empty(n, dtype=torch.int32, device=dev)
            reg = torch.empty(n, dtype=torch.uint8, device=dev)
            _check(_clib.cmg_sdf_plan_copy_outputs(self._h, occ.data_ptr(), sdf.data_ptr(),
                                                   tri.data_ptr(), reg.data_ptr(), st, err, 512),
                   err)
        return sdf, occ, tri, reg

    def backward(self, vertices: torch.Tensor, occ: torch.Tensor, tri: torch.Tensor,
                 reg: torch.Tensor, grad_sdf: torch.Tensor) -> torch.Tensor:
        """dL/d(vertices) (float64, (V, 3)) given dL/d(sdf) per cell (flat)."""
        p = self._points(vertices)
        g = grad_sdf.detach().to(torch.float64).contiguous().view(-1)
        if g.numel() != self.cells:
            raise ValueError("grad_sdf must have one value per cell")
        for t, dt in ((occ, torch.uint8), (tri, torch.int32), (reg, torch.uint8)):
            if t.dtype != dt or t.numel() != self.cells or not t.is_contiguous():
                raise ValueError("checkpoint arrays must come from SDFPlan.forward")
        out = torch.empty((self.npoints, 3), dtype=torch.float64, device=p.device)
        err = _err()
        with torch.cuda.device(p.device):
            _check(_clib.cmg_sdf_plan_backward(self._h, p.data_ptr(), occ.data_ptr(),
                                               tri.data_ptr(), reg.data_ptr(), g.data_ptr(),
                                               out.data_ptr(), _stream(), err, 512), err)
        return out


class _SDF(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vertices: torch.Tensor, plan: SDFPlan):
        sdf, occ, tri, reg = plan.forward(vertices)
        ctx.plan = plan
        ctx.save_for_backward(vertices.detach().to(torch.float64), occ, tri, reg)
        ctx.dtype = vertices.dtype
        return sdf.to(vertices.dtype)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        v, occ, tri, reg = ctx.saved_tensors
        grad = ctx.plan.backward(v, occ, tri, reg, grad_out)
        return grad.to(ctx.dtype), None


def sdf(vertices: torch.Tensor, plan: Optional[SDFPlan] = None, faces=None, grid=None,
        precision: int = PREC_FP64) -> torch.Tensor:
    """Signed distance of every cell of the grid, shape ``(nx, ny, nz)``,
    differentiable in ``vertices`` (``(V, 3)`` CUDA tensor, float32 or float64).
    Give a :class:`SDFPlan` for repeated calls, or ``faces`` and ``grid`` to plan
    this call alone."""
    if plan is None:
        if faces is None or grid is None:
            raise ValueError("give a plan, or faces and grid")
        plan = SDFPlan(vertices, faces, grid, precision=precision)
    nx, ny, nz = plan.dims
    flat = _SDF.apply(vertices, plan)
    return flat.view(nz, ny, nx).permute(2, 1, 0)


def grid_of(corner: Sequence[float], spacing: float, dims: Sequence[int]):
    """The ``grid`` tuple of :class:`SDFPlan`."""
    return (tuple(float(c) for c in corner), float(spacing), tuple(int(d) for d in dims))
