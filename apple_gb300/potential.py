"""External force potential (warp/potential/_ext_force.py:17-90).

W = -sum_i f_i . u_i, grad = -f at the loaded points, Hessian terms zero.
Inside a model the force is folded into the native vertex passes; on its
own it runs as a model without FEM terms.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .fem import Space, WarpPotential, _default_name, check_scalar, check_vec, dtype_code, ptr, stream_ptr
from .region import FORCE, GLOBAL_POINT_ID, mesh_points, point_data


class ExternalForce(WarpPotential):
    def __init__(self, indices, force, *, n_points: int | None = None, name: str | None = None,
                 dtype: torch.dtype = torch.float32):
        self.indices = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1)
        self.force = np.ascontiguousarray(force, dtype=np.float64).reshape(-1, 3)
        if self.indices.shape[0] != self.force.shape[0]:
            raise ValueError("indices and force lengths differ")
        self.n_points = int(n_points if n_points is not None else (self.indices.max() + 1 if self.indices.size else 0))
        self.name = name or _default_name(self)
        self.dtype = dtype
        self._own = None

    @classmethod
    def from_pyvista(cls, obj, **kw) -> "ExternalForce":
        """Point data ``Force`` and ``GlobalPointId`` (_ext_force.py:55-61)."""
        pd = point_data(obj)
        force = np.asarray(pd[FORCE], np.float64)
        if GLOBAL_POINT_ID in pd:
            idx = np.asarray(pd[GLOBAL_POINT_ID])
        else:
            idx = np.arange(mesh_points(obj).shape[0])
        return cls(idx, force, **kw)

    from_mesh = from_pyvista

    def _model(self):
        if self._own is None:
            space = Space(self.n_points, None)
            h = ctypes.c_void_p()
            _lib.call(
                "agb_model_create", space.handle, dtype_code(self.dtype), 0, None, None, None,
                self.indices.shape[0], self.indices.ctypes.data, self.force.ctypes.data, ctypes.byref(h),
            )
            self._own = (space, h)
        return self._own[1]

    def __del__(self):
        own = getattr(self, "_own", None)
        if own is not None and _lib._lib is not None:
            _lib.load().agb_model_destroy(own[1])
        self._own = None

    def fun(self, u: torch.Tensor, output: torch.Tensor) -> None:
        check_vec(u, self.n_points, self.dtype, "u")
        check_scalar(output, "output")
        tmp = torch.empty((1,), dtype=torch.float64, device=u.device)
        _lib.call("agb_model_eval", self._model(), _lib.FUN, ptr(u), None, ptr(tmp), None, None, None, None,
                  stream_ptr(u.device))
        output[:1] += tmp

    def grad(self, u: torch.Tensor, output: torch.Tensor) -> None:
        check_vec(u, self.n_points, self.dtype, "u")
        check_vec(output, self.n_points, self.dtype, "output")
        tmp = torch.empty_like(output)
        _lib.call("agb_model_eval", self._model(), _lib.GRAD, ptr(u), None, None, ptr(tmp), None, None, None,
                  stream_ptr(u.device))
        output += tmp

    jac = grad

    def hess_diag(self, u, output) -> None:  # _ext_force.py:80-82
        pass

    def hess_prod(self, u, p, output) -> None:
        pass

    def hess_quad(self, u, p, output) -> None:
        pass
