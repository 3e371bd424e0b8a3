"""Differentiation of the quasi-static equilibrium with respect to cell materials.

The reference's inverse experiments differentiate ``Forward.step()`` by hand
(exp/2025/09/24/inverse-grin/src/32-inverse.py:223-300): at the converged
u*, solve ``H(u*) lam = dL/du`` on the free DOFs with Jacobi-preconditioned
CG over ``hess_prod``, then pull ``lam`` back to the material arrays through
the backward of the gradient kernel (Warp's tape over the arrays named in
``requires_grad``), ``dL/dtheta = -d(lam . g)/dtheta``.

Here the CG runs on the device inside the PNCG solver that produced u*
(``DeviceSolver.adjoint`` -> ``agb_solver_adjoint``) and the pull-back is
``WarpPotentialFem.grad_param_vjp`` (``agb_fem_grad_param_vjp``).
:class:`MaterialEquilibrium` packages forward + adjoint for one FEM potential
whose per-cell ``mu`` (and ``lambda``) are the parameters -- and, for
:class:`StableNeoHookeanMuscle`, the per-cell ``activation`` (the parameter
of the reference's inverse activation fits) -- and
:class:`EquilibriumFunction` exposes it to ``torch.autograd``.
"""

from __future__ import annotations

import dataclasses
import time

import numpy as np
import torch

from . import meshgen
from .fem import StableNeoHookean, StableNeoHookeanMuscle, WarpPotentialFem
from .forward import Forward, ModelState
from .model import ModelBuilder
from .pncg import PNCG, CgSolution, ConvergenceCriteria, Result, Solution
from .potential import ExternalForce
from .region import FIXED_MASK, FIXED_VALUE, LAMBDA, MU


@dataclasses.dataclass
class AdjointStats:
    forward: Solution
    cg: CgSolution | None = None


class MaterialEquilibrium:
    """u*(mu, lambda) = argmin of the model energy, and its vector-Jacobian product.

    ``mesh`` is a tetrahedral mesh (``points``, ``cells``, ``point_data`` with
    ``FixedMask`` / ``FixedValue``); ``material`` a :class:`WarpPotentialFem`
    subclass; ``force`` an optional (n_points, 3) external force.
    """

    def __init__(self, mesh, material: type[WarpPotentialFem] = StableNeoHookean, *,
                 force: np.ndarray | None = None, dtype: torch.dtype = torch.float32,
                 criteria: ConvergenceCriteria | None = None, cg_rtol: float = 1e-6,
                 cg_max_iter: int = 20000, device: torch.device | str = "cuda"):
        self.points = np.asarray(mesh.points, np.float64)
        self.cells = np.asarray(mesh.cells, np.int32).reshape(-1, 4)
        self.fixed_mask = np.asarray(mesh.point_data[FIXED_MASK], bool).reshape(-1, 3)
        self.fixed_values = np.asarray(mesh.point_data.get(FIXED_VALUE, np.zeros_like(self.points)),
                                       np.float64).reshape(-1, 3)
        self.material = material
        self.force = None if force is None else np.asarray(force, np.float64).reshape(-1, 3)
        self.dtype = dtype
        self.criteria = criteria or ConvergenceCriteria(max_steps=20000)
        self.cg_rtol = cg_rtol
        self.cg_max_iter = cg_max_iter
        self.device = torch.device(device)
        self._state = None  # (potential, solver, u*, model) of the last forward
        self._opt = None
        self._key = None  # the (mu, lambda) the resident model was built with
        self.stats: AdjointStats | None = None
        self.timings: dict[str, float] = {}  # seconds of the last solve() / vjp() phases

    @property
    def n_cells(self) -> int:
        return self.cells.shape[0]

    @property
    def muscle(self) -> bool:
        return issubclass(self.material, StableNeoHookeanMuscle)

    def solve(self, mu, lam=None, activation=None, u0: torch.Tensor | None = None) -> torch.Tensor:
        """Forward: the converged displacement (n_points, 3) for these cell
        materials (``activation`` (n_cells, 6): muscle only), from zero free
        displacement or from ``u0`` (its free components; a warm start, as an
        optimisation loop takes from its previous iterate).  When only the
        activation changed since the last call, the resident device model is
        kept (new activation records, same tiles and solver)."""
        t0 = time.perf_counter()
        act = None
        if self.muscle:
            act = np.zeros((self.n_cells, 6)) if activation is None else \
                np.asarray(torch.as_tensor(activation).detach().cpu(), np.float64).reshape(self.n_cells, 6)
        elif activation is not None:
            raise ValueError("activation is a muscle parameter")
        key = (np.asarray(torch.as_tensor(mu).detach().cpu(), np.float64).tobytes(),
               None if lam is None else np.asarray(torch.as_tensor(lam).detach().cpu(), np.float64).tobytes())
        if act is not None and self._state is not None and self._key == key:
            pot, sv, _, model = self._state
            pot.set_activation(act)
            opt = self._opt
            fwd = Forward(model, opt, self._initial_state(model, u0))
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            sol = fwd.step()
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            self._state = (pot, sv, fwd.state.u, model)
            self.stats = AdjointStats(sol)
            self.timings = {"build": t1 - t0, "forward": t2 - t1}
            return fwd.state.u
        mesh = meshgen.TetMesh(self.points, self.cells)
        mesh.cell_data[MU] = np.asarray(torch.as_tensor(mu).detach().cpu(), np.float64)
        if lam is not None:
            mesh.cell_data[LAMBDA] = np.asarray(torch.as_tensor(lam).detach().cpu(), np.float64)
        if act is not None:
            mesh.cell_data["activation"] = act
        mesh.point_data[FIXED_MASK] = self.fixed_mask
        mesh.point_data[FIXED_VALUE] = self.fixed_values
        pot = self.material.from_pyvista(mesh, dtype=self.dtype)
        b = ModelBuilder(dtype=self.dtype)
        b.add_vertices(mesh)
        b.add_fixed(mesh)
        b.add_potential(pot)
        if self.force is not None:
            fm = meshgen.TetMesh(self.points, self.cells)
            fm.point_data["Force"] = self.force
            fm.point_data["GlobalPointId"] = np.arange(self.points.shape[0])
            b.add_potential(ExternalForce.from_pyvista(fm, dtype=self.dtype))
        model = b.finalize()
        opt = PNCG(self.criteria)
        fwd = Forward(model, opt, self._initial_state(model, u0))
        opt.solver(fwd.problem)  # device set-up outside the timed solve
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        sol = fwd.step()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        u = fwd.state.u
        self._state = (pot, opt.solver(fwd.problem), u, model)
        self._opt = opt
        self._key = key
        self.stats = AdjointStats(sol)
        self.timings = {"build": t1 - t0, "forward": t2 - t1}
        return u

    def _initial_state(self, model, u0):
        if u0 is None:
            return None
        dm = model.dof_map
        u0 = u0.to(dtype=model.dtype, device=dm.free_indices.device).reshape(-1, 3)
        return ModelState(u=dm.to_full(dm.to_free(u0)))

    def vjp(self, grad_u: torch.Tensor) -> dict:
        """dL/dmu (and dL/dlambda; dL/dactivation for the muscle) per cell for
        dL/du = grad_u at the last forward's u*."""
        if self._state is None:
            raise RuntimeError("call solve() first")
        pot, sv, u, _ = self._state
        rhs = grad_u.to(self.dtype).to(u.device).contiguous()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lam, cg = sv.adjoint(rhs, rtol=self.cg_rtol, max_iter=self.cg_max_iter)
        self.stats = dataclasses.replace(self.stats, cg=cg)
        if cg.result not in (Result.PRIMARY_SUCCESS,):
            raise RuntimeError(f"adjoint CG did not converge: {cg}")
        out = pot.grad_param_vjp(u, lam)
        torch.cuda.synchronize()
        self.timings["adjoint"] = time.perf_counter() - t0
        return {k: -v for k, v in out.items()}


class EquilibriumFunction(torch.autograd.Function):
    """``u = EquilibriumFunction.apply(mu, lam, problem[, activation])``: the
    converged displacement as a differentiable function of the per-cell
    materials (``lam`` may be None for ARAP; ``activation`` (n_cells, 6) for
    the muscle)."""

    @staticmethod
    def forward(ctx, mu, lam, problem: MaterialEquilibrium, activation=None):
        u = problem.solve(mu, lam, activation)
        ctx.problem = problem
        ctx.has_lam = lam is not None
        ctx.has_act = activation is not None
        ctx.mu_dtype = mu.dtype
        ctx.mu_device = mu.device
        return u.to(mu.dtype)

    @staticmethod
    def backward(ctx, grad_u):
        g = ctx.problem.vjp(grad_u)
        cast = lambda t: t.to(dtype=ctx.mu_dtype, device=ctx.mu_device)  # noqa: E731
        dmu = cast(g["mu"])
        dlam = cast(g["lambda"]) if ctx.has_lam and "lambda" in g else None
        dact = cast(g["activation"]) if ctx.has_act and "activation" in g else None
        return dmu, dlam, None, dact
