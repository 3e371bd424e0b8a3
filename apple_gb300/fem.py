"""FEM potentials: ``Arap`` and ``StableNeoHookean``.

Mirror of ``WarpPotentialFem`` (warp/fem/_base.py:39-194) and its materials
(warp/fem/_arap.py:79-125, warp/fem/_stable_neo_hookean.py:231-279).  The
five methods take CUDA tensors of shape (n_points, 3) and ACCUMULATE into
``output`` as the reference does; scalar outputs are float64 tensors of
shape (1,).  Every method runs the native sm_103a kernels of
``libapple_gb300.so`` through its C ABI; there is no other code path.
"""

from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch

from . import _lib
from .region import ACTIVATION, FRACTION, LAMBDA, MU, Region, cell_data

_counter: dict[str, int] = {}


def _default_name(obj) -> str:
    # common/_potential_name.py:6-16
    cls = type(obj).__name__
    k = _counter.get(cls, 0)
    _counter[cls] = k + 1
    return f"{cls}{k}"


def dtype_code(dtype: torch.dtype) -> int:
    if dtype == torch.float32:
        return _lib.F32
    if dtype == torch.float64:
        return _lib.F64
    raise TypeError(f"unsupported dtype {dtype}: use torch.float32 or torch.float64")


def stream_ptr(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def check_vec(t: torch.Tensor, n_points: int, dtype: torch.dtype, name: str) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} has dtype {t.dtype}, the potential computes in {dtype}")
    if tuple(t.shape) != (n_points, 3) or not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous with shape ({n_points}, 3), got {tuple(t.shape)}")
    return t


def check_scalar(t: torch.Tensor, name: str) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64 or t.numel() < 1:
        raise TypeError(f"{name} must be a CUDA float64 tensor with at least one element")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return t


class Space:
    """A vertex set with its device order (``agb_space``)."""

    def __init__(self, n_points: int, points: np.ndarray | None):
        h = ctypes.c_void_p()
        pts = None if points is None else np.ascontiguousarray(points, dtype=np.float64)
        _lib.call("agb_space_create", int(n_points), None if pts is None else pts.ctypes.data, ctypes.byref(h))
        self.handle = h
        self.n_points = int(n_points)

    def order(self) -> np.ndarray:
        out = np.empty(self.n_points, np.int32)
        _lib.call("agb_space_order", self.handle, out.ctypes.data)
        return out

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib.load().agb_space_destroy(self.handle)
            self.handle = None


class _Owned:
    """One C handle, destroyed with this wrapper (``destroy``: the C call)."""

    def __init__(self, handle: ctypes.c_void_p, destroy: str):
        self.handle = handle
        self._destroy = destroy

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            getattr(_lib.load(), self._destroy)(self.handle)
            self.handle = None


class WarpPotential:
    """The energy-term interface of warp/model/_potential.py:9-32: every
    method accumulates into ``output`` (the caller zeroes it); the base
    raises ``NotImplementedError`` like the reference's."""

    def fun(self, u: torch.Tensor, output: torch.Tensor) -> None:
        raise NotImplementedError

    def grad(self, u: torch.Tensor, output: torch.Tensor) -> None:
        raise NotImplementedError

    def hess_diag(self, u: torch.Tensor, output: torch.Tensor) -> None:
        raise NotImplementedError

    def hess_prod(self, u: torch.Tensor, p: torch.Tensor, output: torch.Tensor) -> None:
        raise NotImplementedError

    def hess_quad(self, u: torch.Tensor, p: torch.Tensor, output: torch.Tensor) -> None:
        raise NotImplementedError


class WarpPotentialFem(WarpPotential):
    """A tetrahedral FEM energy term on the GPU."""

    material: int = -1

    def __init__(
        self,
        cells: np.ndarray,
        mu: np.ndarray,
        lam: np.ndarray | None = None,
        *,
        points: np.ndarray | None = None,
        dhdX: np.ndarray | None = None,
        dV: np.ndarray | None = None,
        fraction: np.ndarray | None = None,
        n_points: int | None = None,
        name: str | None = None,
        dtype: torch.dtype = torch.float32,
        tile_elems: int = 0,
        requires_grad=(),
    ):
        self.cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 4)
        n_cells = self.cells.shape[0]
        self.mu = np.ascontiguousarray(np.broadcast_to(np.asarray(mu, np.float64), (n_cells,)))
        self.lam = None if lam is None else np.ascontiguousarray(np.broadcast_to(np.asarray(lam, np.float64), (n_cells,)))
        self.points = None if points is None else np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        self.dhdX = None if dhdX is None else np.ascontiguousarray(dhdX, dtype=np.float64).reshape(n_cells, 4, 3)
        self.dV = None if dV is None else np.ascontiguousarray(dV, dtype=np.float64).reshape(n_cells)
        self.fraction = None if fraction is None else np.ascontiguousarray(fraction, dtype=np.float64).reshape(n_cells)
        if n_points is None:
            n_points = self.points.shape[0] if self.points is not None else int(self.cells.max()) + 1
        self.n_points = int(n_points)
        self.name = name or _default_name(self)
        self.dtype = dtype
        self.tile_elems = int(tile_elems)
        self.requires_grad = tuple(requires_grad)
        self._own = None  # (space, owned handle) for standalone use
        # one device copy per space, destroyed when its space goes
        self._by_space: weakref.WeakKeyDictionary[Space, _Owned] = weakref.WeakKeyDictionary()

    # -- construction (warp/fem/_base.py:78-111) -------------------------------
    @classmethod
    def from_region(cls, region: Region, *, requires_grad=(), name=None, dtype=torch.float32, **kw):
        if region.dhdX is None:
            region.compute_grad()
        cd = region.cell_data
        mu = np.asarray(cd[MU], np.float64)
        lam = np.asarray(cd[LAMBDA], np.float64) if LAMBDA in cd else None
        frac = np.asarray(cd[FRACTION], np.float64) if FRACTION in cd else None
        n_points = int(region.cells_global.max()) + 1 if region.cells_global.size else 0
        pts = None
        if n_points == region.points.shape[0]:
            pts = region.points
        else:  # global ids beyond this mesh: place its points at their global ids
            pts = np.zeros((n_points, 3))
            pts[region.cells_global.reshape(-1)] = region.points[region.cells_local.reshape(-1)]
        return cls(
            region.cells_global, mu, lam, points=pts, dhdX=region.dhdX[:, 0], dV=region.dV[:, 0],
            fraction=frac, n_points=n_points, name=name, dtype=dtype, requires_grad=requires_grad, **kw,
        )

    @classmethod
    def from_pyvista(cls, mesh, **kw):
        return cls.from_region(Region.from_pyvista(mesh, grad=True), **kw)

    from_mesh = from_pyvista

    # -- device objects --------------------------------------------------------
    def _create(self, space: Space) -> ctypes.c_void_p:
        h = ctypes.c_void_p()
        arr = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        _lib.call(
            "agb_fem_create", space.handle, self.material, dtype_code(self.dtype), self.cells.shape[0],
            self.cells.ctypes.data, arr(self.points) if self.points is not None and self.points.shape[0] == space.n_points else None,
            arr(self.dhdX), arr(self.dV), arr(self.fraction), self.mu.ctypes.data,
            arr(self.lam),
            self.tile_elems, ctypes.byref(h),
        )
        return h

    def on_space(self, space: Space) -> ctypes.c_void_p:
        """The device potential over ``space`` (created once per space)."""
        owned = self._by_space.get(space)
        if owned is None:
            owned = self._by_space[space] = _Owned(self._create(space), "agb_fem_destroy")
        return owned.handle

    def _standalone(self) -> ctypes.c_void_p:
        if self._own is None:
            space = Space(self.n_points, self.points)
            self._own = (space, _Owned(self._create(space), "agb_fem_destroy"))
        return self._own[1].handle

    def _handles(self) -> list[ctypes.c_void_p]:
        """Every device copy of this potential."""
        out = [o.handle for o in list(self._by_space.values())]
        return out + ([self._own[1].handle] if self._own is not None else [])

    def info(self) -> tuple[int, int]:
        nt, ntv = ctypes.c_int32(), ctypes.c_int32()
        _lib.call("agb_fem_info", self._standalone(), ctypes.byref(nt), ctypes.byref(ntv))
        return nt.value, ntv.value

    def stored_cells(self) -> tuple[np.ndarray, int]:
        """(cells as stored after reorder / tiling / colouring, in the caller's
        cell order and point ids; hash of the tile and colour plan)."""
        out = np.empty((self.cells.shape[0], 4), np.int32)
        h = ctypes.c_uint32()
        _lib.call("agb_fem_cells", self._standalone(), out.ctypes.data, ctypes.byref(h))
        return out, h.value

    # -- WarpPotential surface (warp/model/_potential.py:19-32) ----------------
    def fun(self, u: torch.Tensor, output: torch.Tensor) -> None:
        check_vec(u, self.n_points, self.dtype, "u")
        check_scalar(output, "output")
        _lib.call("agb_fem_fun", self._standalone(), ptr(u), ptr(output), stream_ptr(u.device))

    def grad(self, u: torch.Tensor, output: torch.Tensor) -> None:
        check_vec(u, self.n_points, self.dtype, "u")
        check_vec(output, self.n_points, self.dtype, "output")
        _lib.call("agb_fem_grad", self._standalone(), ptr(u), ptr(output), stream_ptr(u.device))

    jac = grad

    def hess_diag(self, u: torch.Tensor, output: torch.Tensor) -> None:
        check_vec(u, self.n_points, self.dtype, "u")
        check_vec(output, self.n_points, self.dtype, "output")
        _lib.call("agb_fem_hess_diag", self._standalone(), ptr(u), ptr(output), stream_ptr(u.device))

    def hess_prod(self, u: torch.Tensor, p: torch.Tensor, output: torch.Tensor) -> None:
        check_vec(u, self.n_points, self.dtype, "u")
        p = check_vec(p.to(self.dtype), self.n_points, self.dtype, "p")
        check_vec(output, self.n_points, self.dtype, "output")
        _lib.call("agb_fem_hess_prod", self._standalone(), ptr(u), ptr(p), ptr(output), stream_ptr(u.device))

    def hess_quad(self, u: torch.Tensor, p: torch.Tensor, output: torch.Tensor) -> None:
        check_vec(u, self.n_points, self.dtype, "u")
        p = check_vec(p.to(self.dtype), self.n_points, self.dtype, "p")
        check_scalar(output, "output")
        _lib.call("agb_fem_hess_quad", self._standalone(), ptr(u), ptr(p), ptr(output), stream_ptr(u.device))

    def grad_param_vjp(self, u: torch.Tensor, w: torch.Tensor) -> dict:
        """Backward of ``grad`` on the cell materials: ``{"mu": d(w.grad(u))/d mu,
        "lambda": d(w.grad(u))/d lambda}`` per cell (what Warp's tape gives for the
        arrays in ``requires_grad``, warp/fem/_base.py:80-117)."""
        check_vec(u, self.n_points, self.dtype, "u")
        w = check_vec(w.to(self.dtype), self.n_points, self.dtype, "w")
        n = self.cells.shape[0]
        dmu = torch.zeros(n, dtype=self.dtype, device=u.device)
        dlam = torch.zeros(n, dtype=self.dtype, device=u.device)
        _lib.call("agb_fem_grad_param_vjp", self._standalone(), ptr(u), ptr(w), ptr(dmu), ptr(dlam),
                  stream_ptr(u.device))
        out = {"mu": dmu}
        if self.material != _lib.ARAP:
            out["lambda"] = dlam
        return out

    def eval(self, u: torch.Tensor, p: torch.Tensor | None = None, *, fun=False, grad=False,
             hess_diag=False, hess_prod=False, hess_quad=False) -> dict:
        """Fused: the requested quantities from one pass over the mesh (new tensors)."""
        check_vec(u, self.n_points, self.dtype, "u")
        flags = (_lib.FUN * fun) | (_lib.GRAD * grad) | (_lib.HESS_DIAG * hess_diag) | \
            (_lib.HESS_PROD * hess_prod) | (_lib.HESS_QUAD * hess_quad)
        if (hess_prod or hess_quad):
            if p is None:
                raise ValueError("p is required for hess_prod / hess_quad")
            p = check_vec(p.to(self.dtype), self.n_points, self.dtype, "p")
        out = {}
        z = lambda: torch.zeros((self.n_points, 3), dtype=self.dtype, device=u.device)  # noqa: E731
        s = lambda: torch.zeros((1,), dtype=torch.float64, device=u.device)  # noqa: E731
        if fun:
            out["fun"] = s()
        if grad:
            out["grad"] = z()
        if hess_diag:
            out["hess_diag"] = z()
        if hess_prod:
            out["hess_prod"] = z()
        if hess_quad:
            out["hess_quad"] = s()
        _lib.call(
            "agb_fem_eval", self._standalone(), flags, ptr(u), ptr(p), ptr(out.get("fun")), ptr(out.get("grad")),
            ptr(out.get("hess_diag")), ptr(out.get("hess_prod")), ptr(out.get("hess_quad")), stream_ptr(u.device),
        )
        return out


class Arap(WarpPotentialFem):
    """Psi = mu/2 ||F - R||^2 (warp/fem/_arap.py:17-28); cell data ``mu``."""

    material = _lib.ARAP


class StableNeoHookean(WarpPotentialFem):
    """Psi = mu/2 (I2 - 3) - mu (J - 1) + lambda/2 (J - 1)^2
    (warp/fem/_stable_neo_hookean.py:17-27); cell data ``mu`` and ``lambda``."""

    material = _lib.STABLE_NEO_HOOKEAN


def _activation_array(activation, n_cells: int) -> np.ndarray:
    """(n_cells, 6) float64 from None (zeros), one 6-vector, or per-cell rows."""
    if activation is None:
        return np.zeros((n_cells, 6))
    a = np.asarray(activation, np.float64)
    if a.shape == (6,):
        a = np.broadcast_to(a, (n_cells, 6))
    return np.ascontiguousarray(a.reshape(n_cells, 6)).copy()


class StableNeoHookeanMuscle(WarpPotentialFem):
    """Stable Neo-Hookean of G = F A with the per-cell activation
    A = I + [[a0, a3, a4], [a3, a1, a5], [a4, a5, a2]]
    (warp/fem/_stable_neo_hookean_muscle.py:18-46, func/_misc.py:48-53);
    cell data ``mu``, ``lambda`` and ``activation`` (n_cells, 6)."""

    material = _lib.STABLE_NEO_HOOKEAN_MUSCLE

    def __init__(self, cells, mu, lam=None, *, activation=None, **kw):
        super().__init__(cells, mu, lam, **kw)
        n = self.cells.shape[0]
        self.activation = _activation_array(activation, n)

    @classmethod
    def from_region(cls, region: Region, **kw):
        cd = region.cell_data
        key = "activation" if "activation" in cd else ACTIVATION
        if "activation" not in kw:
            kw["activation"] = np.asarray(cd[key], np.float64).reshape(-1, 6) if key in cd else None
        return super().from_region(region, **kw)

    def _create(self, space: Space) -> ctypes.c_void_p:
        h = super()._create(space)
        try:
            _lib.call("agb_fem_set_activation", h, self.activation.ctypes.data)
        except BaseException:
            _lib.load().agb_fem_destroy(h)
            raise
        return h

    def set_activation(self, activation) -> None:
        """Replace the per-cell activation on every device copy of this potential.
        A solver whose model has this as its only FEM potential sees the new
        records at its next launch; a solver over several potentials copied
        the records when it was created and needs to be built again."""
        self.activation = _activation_array(activation, self.cells.shape[0])
        for h in self._handles():
            _lib.call("agb_fem_set_activation", h, self.activation.ctypes.data)

    def grad_param_vjp(self, u: torch.Tensor, w: torch.Tensor) -> dict:
        """As :meth:`WarpPotentialFem.grad_param_vjp`, plus ``"activation"``:
        d(w.grad(u))/d activation, (n_cells, 6)."""
        out = super().grad_param_vjp(u, w)
        w = check_vec(w.to(self.dtype), self.n_points, self.dtype, "w")
        da = torch.zeros((self.cells.shape[0], 6), dtype=self.dtype, device=u.device)
        _lib.call("agb_fem_grad_activation_vjp", self._standalone(), ptr(u), ptr(w), ptr(da), stream_ptr(u.device))
        out["activation"] = da
        return out


def with_lame(mesh, mu, lam=None):
    """Write scalar or per-cell Lame parameters into ``mesh.cell_data``."""
    from .region import mesh_cells

    n = mesh_cells(mesh).shape[0]
    cd = cell_data(mesh)
    cd[MU] = np.broadcast_to(np.asarray(mu, np.float64), (n,)).copy()
    if lam is not None:
        cd[LAMBDA] = np.broadcast_to(np.asarray(lam, np.float64), (n,)).copy()
    return mesh
