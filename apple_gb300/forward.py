"""Quasi-static forward solve (forward/_forward.py, forward/_problem.py)."""

from __future__ import annotations

import dataclasses
import functools

import torch

from .model import DofMap, DofMapBuilder, Model, ModelBuilder
from .pncg import PNCG, ConvergenceCriteria, LineSearch, Solution

# the names of liblaf.apple.forward (forward/__init__.pyi)
__all__ = ["DofMap", "DofMapBuilder", "Forward", "ForwardProblem", "Model", "ModelBuilder", "ModelState"]


@dataclasses.dataclass
class ModelState:
    u: torch.Tensor  # full displacement (n_points, 3)


class ForwardProblem:
    """Free-DOF problem over a model (forward/_problem.py:18-59)."""

    State = ModelState

    def __init__(self, model: Model):
        self.model = model

    def before_trial(self, state: ModelState, u: torch.Tensor) -> ModelState:
        return dataclasses.replace(state, u=self.model.dof_map.to_full(u))

    def max_step_size(self, state: ModelState, p: torch.Tensor) -> torch.Tensor:
        return torch.ones((), dtype=torch.float64, device=p.device)  # no collision term

    def fun(self, state: ModelState) -> torch.Tensor:
        return self.model.fun(state.u)

    def grad(self, state: ModelState) -> torch.Tensor:
        return self.model.dof_map.to_free_grad(self.model.grad(state.u))

    def hess_diag(self, state: ModelState) -> torch.Tensor:
        return self.model.dof_map.to_free_hess_diag(self.model.hess_diag(state.u))

    def hess_prod(self, state: ModelState, p: torch.Tensor) -> torch.Tensor:
        p_full = self.model.dof_map.to_full_grad(p)
        return self.model.dof_map.to_free_grad(self.model.hess_prod(state.u, p_full))

    def hess_quad(self, state: ModelState, p: torch.Tensor) -> torch.Tensor:
        return self.model.hess_quad(state.u, self.model.dof_map.to_full_grad(p))


class Forward:
    """forward/_forward.py:18-56: ``step()`` minimises the total energy."""

    def __init__(self, model: Model, optimizer: PNCG | None = None, state: ModelState | None = None):
        self.model = model
        self.optimizer = optimizer or PNCG(criteria=ConvergenceCriteria(max_steps=1500), line_search=LineSearch())
        if state is None:
            dm = model.dof_map
            free = torch.zeros(dm.n_free, dtype=model.dtype, device=dm.free_indices.device)
            state = ModelState(u=dm.to_full(free))
        self.state = state

    @property
    def free(self) -> torch.Tensor:
        return self.model.dof_map.to_free(self.state.u)

    @functools.cached_property
    def problem(self) -> ForwardProblem:
        return ForwardProblem(self.model)

    def step(self) -> Solution:
        solution, self.state = self.optimizer.minimize(self.problem, self.state, self.free)
        return solution
