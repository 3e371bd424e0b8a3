"""Models: the sum of energy terms over one vertex set, with fixed DOFs.

* ``DofMap`` / ``DofMapBuilder``  -- forward/dof_map/_dof_map.py:10-49, _builder.py:13-64
* ``WarpModel``                   -- warp/model/_model.py:9-36 (zero, then accumulate)
* ``Model``                       -- forward/_model.py:14-74 (pure functions of u)
* ``ModelBuilder``                -- forward/_builder.py:12-40

The device model (``agb_model``) holds every FEM term, the fixed mask and
values, and the external forces; one call evaluates all of them.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .fem import Space, WarpPotentialFem, check_vec, dtype_code, ptr, stream_ptr
from .potential import ExternalForce
from .region import FIXED_MASK, FIXED_VALUE, GLOBAL_POINT_ID, mesh_points, point_data


class DofMap:
    """Free/fixed DOF gather and scatter over the flattened (n_points*3) vector
    (forward/dof_map/_dof_map.py:10-50).  Each map is one kernel of the C
    library (``agb_dof_to_free`` / ``agb_dof_to_full``) on the caller's
    current stream; ``to_full`` gathers through a full-length slot map (the
    DOF's free index, or -1 for a fixed DOF) with the fixed values as fill."""

    def __init__(self, n_points: int, fixed_mask: np.ndarray, fixed_values: np.ndarray, *, dim: int = 3,
                 device=None, dtype=torch.float32):
        self.dim = dim
        self.n_points = int(n_points)
        self.fixed_mask = np.asarray(fixed_mask, bool).reshape(n_points, dim)
        self.fixed_values_full = np.asarray(fixed_values, np.float64).reshape(n_points, dim)
        device = device or torch.device("cuda", torch.cuda.current_device())
        flat = self.fixed_mask.reshape(-1)
        fixed = np.flatnonzero(flat)
        free = np.flatnonzero(~flat)
        self.fixed_indices = torch.as_tensor(fixed, device=device)
        self.free_indices = torch.as_tensor(free, device=device)
        self.fixed_values = torch.as_tensor(self.fixed_values_full.reshape(-1)[fixed], dtype=dtype, device=device)
        slot = np.full(flat.size, -1, np.int32)
        slot[free] = np.arange(free.size, dtype=np.int32)
        self.slot = torch.as_tensor(slot, device=device)
        fill = np.zeros(flat.size)
        fill[fixed] = self.fixed_values_full.reshape(-1)[fixed]
        self._fill64 = fill
        self._fill: dict[torch.dtype, torch.Tensor] = {}
        self.dtype = dtype

    @property
    def n_fixed(self) -> int:
        return int(self.fixed_indices.numel())

    @property
    def n_free(self) -> int:
        return int(self.free_indices.numel())

    @property
    def n_full(self) -> int:
        return self.n_points * self.dim

    def _fill_for(self, dtype: torch.dtype) -> torch.Tensor:
        f = self._fill.get(dtype)
        if f is None:
            f = self._fill[dtype] = torch.as_tensor(self._fill64, dtype=dtype, device=self.slot.device)
        return f

    def _check(self, t: torch.Tensor, n: int, name: str) -> torch.Tensor:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a tensor")
        if t.numel() != n:
            raise ValueError(f"{name} has {t.numel()} entries, expected {n}")
        if t.device != self.slot.device:
            raise ValueError(f"{name} is on {t.device}, the map on {self.slot.device}")
        dtype_code(t.dtype)  # float32 / float64 only
        return t.reshape(-1).contiguous()

    # A map built on the host (device="cpu", for host-side model assembly)
    # indexes host tensors directly; a map on a GPU runs the kernels.
    def to_free(self, full: torch.Tensor) -> torch.Tensor:
        full = self._check(full, self.n_full, "full")
        if not full.is_cuda:
            return full[self.free_indices]
        out = torch.empty(self.n_free, dtype=full.dtype, device=full.device)
        _lib.call("agb_dof_to_free", dtype_code(full.dtype), self.n_free, ptr(self.free_indices), ptr(full),
                  ptr(out), stream_ptr(full.device))
        return out

    to_free_grad = to_free
    to_free_hess_diag = to_free

    def _to_full(self, free: torch.Tensor, fill: bool) -> torch.Tensor:
        free = self._check(free, self.n_free, "free")
        f = self._fill_for(free.dtype) if fill else None
        if not free.is_cuda:
            out = f.clone() if f is not None else torch.zeros(self.n_full, dtype=free.dtype)
            out[self.free_indices] = free
            return out.reshape(self.n_points, self.dim)
        out = torch.empty((self.n_points, self.dim), dtype=free.dtype, device=free.device)
        _lib.call("agb_dof_to_full", dtype_code(free.dtype), self.n_full, ptr(self.slot), ptr(free), ptr(f), ptr(out),
                  stream_ptr(free.device))
        return out

    def to_full(self, free: torch.Tensor) -> torch.Tensor:
        return self._to_full(free, True)

    def to_full_grad(self, free: torch.Tensor) -> torch.Tensor:
        return self._to_full(free, False)


class DofMapBuilder:
    def __init__(self, dim: int = 3):
        self.dim = dim
        self.fixed_mask = np.zeros((0, dim), bool)
        self.full_values = np.zeros((0, dim))
        self.points = np.zeros((0, dim))

    @property
    def n_points(self) -> int:
        return self.fixed_mask.shape[0]

    def add_vertices(self, obj) -> None:
        """Assigns ``GlobalPointId`` (forward/dof_map/_builder.py:41-50)."""
        pts = mesh_points(obj)
        point_data(obj)[GLOBAL_POINT_ID] = np.arange(self.n_points, self.n_points + pts.shape[0])
        self.fixed_mask = np.pad(self.fixed_mask, ((0, pts.shape[0]), (0, 0)), constant_values=False)
        self.full_values = np.pad(self.full_values, ((0, pts.shape[0]), (0, 0)), constant_values=0.0)
        self.points = np.concatenate([self.points, pts], axis=0)

    def add_fixed(self, obj) -> None:
        pd = point_data(obj)
        gid = np.asarray(pd[GLOBAL_POINT_ID])
        self.fixed_mask[gid] = np.asarray(pd[FIXED_MASK], bool).reshape(-1, self.dim)
        self.full_values[gid] = np.asarray(pd[FIXED_VALUE], np.float64).reshape(-1, self.dim)

    def finalize(self, dtype=torch.float32, device=None) -> DofMap:
        return DofMap(self.n_points, self.fixed_mask, self.full_values, dim=self.dim, device=device, dtype=dtype)


class WarpModel:
    """Sum of potentials on one space; methods zero ``output`` and accumulate
    every term (warp/model/_model.py:13-36), in one device call."""

    def __init__(self, potentials, n_points: int, points: np.ndarray | None = None,
                 fixed_mask=None, fixed_values=None, dtype=torch.float32):
        self.potentials = dict(potentials) if not isinstance(potentials, dict) else potentials
        self.n_points = int(n_points)
        self.dtype = dtype
        self.space = Space(self.n_points, points)
        fems = [p for p in self.potentials.values() if isinstance(p, WarpPotentialFem)]
        forces = [p for p in self.potentials.values() if isinstance(p, ExternalForce)]
        for p in self.potentials.values():
            if not isinstance(p, (WarpPotentialFem, ExternalForce)):
                raise TypeError(f"unsupported potential {type(p).__name__}")
            if p.dtype != dtype:
                raise TypeError(f"potential {p.name} computes in {p.dtype}, the model in {dtype}")
        self.fems = fems
        handles = (ctypes.c_void_p * max(1, len(fems)))(*[p.on_space(self.space).value for p in fems])
        idx = np.concatenate([f.indices for f in forces]) if forces else np.zeros(0, np.int32)
        frc = np.concatenate([f.force for f in forces]) if forces else np.zeros((0, 3))
        idx = np.ascontiguousarray(idx, np.int32)
        frc = np.ascontiguousarray(frc, np.float64)
        mask = None if fixed_mask is None else np.ascontiguousarray(np.asarray(fixed_mask, np.uint8).reshape(-1, 3))
        vals = None if fixed_values is None else np.ascontiguousarray(np.asarray(fixed_values, np.float64).reshape(-1, 3))
        h = ctypes.c_void_p()
        _lib.call(
            "agb_model_create", self.space.handle, dtype_code(dtype), len(fems), handles,
            None if mask is None else mask.ctypes.data, None if vals is None else vals.ctypes.data,
            idx.shape[0], idx.ctypes.data if idx.size else None, frc.ctypes.data if frc.size else None,
            ctypes.byref(h),
        )
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib.load().agb_model_destroy(self.handle)
            self.handle = None

    def _eval(self, flags, u, p=None, energy=None, grad=None, diag=None, prod=None, quad=None):
        check_vec(u, self.n_points, self.dtype, "u")
        if p is not None:
            p = check_vec(p.to(self.dtype).contiguous(), self.n_points, self.dtype, "p")
        _lib.call("agb_model_eval", self.handle, flags, ptr(u), ptr(p), ptr(energy), ptr(grad), ptr(diag),
                  ptr(prod), ptr(quad), stream_ptr(u.device))

    def fun(self, u, output) -> None:
        self._eval(_lib.FUN, u, energy=output)

    def grad(self, u, output) -> None:
        self._eval(_lib.GRAD, u, grad=output)

    def hess_diag(self, u, output) -> None:
        self._eval(_lib.HESS_DIAG, u, diag=output)

    def hess_prod(self, u, p, output) -> None:
        self._eval(_lib.HESS_PROD, u, p, prod=output)

    def hess_quad(self, u, p, output) -> None:
        self._eval(_lib.HESS_QUAD, u, p, quad=output)


class Model:
    """Pure functions of the full displacement (forward/_model.py:46-74)."""

    def __init__(self, dof_map: DofMap, warp_model: WarpModel):
        self.dof_map = dof_map
        self.warp_model = warp_model
        self.collision = None

    @property
    def dim(self) -> int:
        return self.dof_map.dim

    @property
    def n_fixed(self) -> int:
        return self.dof_map.n_fixed

    @property
    def n_free(self) -> int:
        return self.dof_map.n_free

    @property
    def n_full(self) -> int:
        return self.dof_map.n_full

    @property
    def n_points(self) -> int:
        return self.dof_map.n_points

    @property
    def dtype(self):
        return self.warp_model.dtype

    def _vec(self, u):
        return torch.empty((self.n_points, 3), dtype=self.dtype, device=u.device)

    def fun(self, u: torch.Tensor) -> torch.Tensor:
        out = torch.empty((1,), dtype=torch.float64, device=u.device)
        self.warp_model.fun(u, out)
        return out[0]

    def grad(self, u):
        out = self._vec(u)
        self.warp_model.grad(u, out)
        return out

    jac = grad

    def hess_diag(self, u):
        out = self._vec(u)
        self.warp_model.hess_diag(u, out)
        return out

    def hess_prod(self, u, p):
        out = self._vec(u)
        self.warp_model.hess_prod(u, p, out)
        return out

    def hess_quad(self, u, p) -> torch.Tensor:
        out = torch.empty((1,), dtype=torch.float64, device=u.device)
        self.warp_model.hess_quad(u, p, out)
        return out[0]

    def init(self):
        from .forward import ModelState

        return ModelState(u=self.dof_map.to_full(torch.zeros(self.n_free, dtype=self.dtype,
                                                             device=self.dof_map.free_indices.device)))


class ModelBuilder:
    """forward/_builder.py:12-40."""

    def __init__(self, dtype: torch.dtype = torch.float32):
        self.dof = DofMapBuilder()
        self.potentials: list = []
        self.collision = None
        self.dtype = dtype

    def add_vertices(self, obj) -> None:
        self.dof.add_vertices(obj)

    def add_fixed(self, obj) -> None:
        self.dof.add_fixed(obj)

    def add_potential(self, potential) -> None:
        if potential.dtype != self.dtype:
            raise TypeError(f"potential {potential.name} computes in {potential.dtype}, the builder in {self.dtype}")
        self.potentials.append(potential)

    def finalize(self) -> Model:
        if self.collision is not None:
            raise NotImplementedError("collision (ipctk) is not part of the GPU path")
        dof_map = self.dof.finalize(dtype=self.dtype)
        n = self.dof.n_points
        for p in self.potentials:
            if p.n_points != n:
                p.n_points = n
        wm = WarpModel({p.name: p for p in self.potentials}, n, self.dof.points,
                       self.dof.fixed_mask, self.dof.full_values, dtype=self.dtype)
        return Model(dof_map, wm)
