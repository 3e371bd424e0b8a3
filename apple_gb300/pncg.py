"""PNCG optimizer front end (the ``liblaf.peach.optim.PNCG`` surface used by
forward/_forward.py:22-30 and exp/2026/05/06/toy/src/
20-ext-force-stable-neo-hookean-collision.py:207-251).

The iteration runs on the device (``agb_solver``: fused element passes and a
CUDA-graph while loop); this module only moves state in and out.  Iteration:
Jacobi preconditioner with the mean fill for zero entries, Dai-Kou beta with
resets (non-finite, |beta| > 10, first step, after a rejected line search),
steepest-descent fallback for non-descent directions, first trial
alpha_0 = overstep * (-g.p / p.Hp) with the proxy's guards, Armijo backtracking
with c = 1e-4 and up to 8 halvings
(benches/bench_pncg_branching_backends.py:254-456, 606-679).
"""

from __future__ import annotations

import ctypes
import dataclasses
import enum
import weakref

import torch

from . import _lib
from .fem import ptr, stream_ptr


class Result(enum.IntEnum):
    PRIMARY_SUCCESS = _lib.PRIMARY_SUCCESS
    MAX_STEPS_REACHED = _lib.MAX_STEPS_REACHED
    LINE_SEARCH_FAILED = _lib.LINE_SEARCH_FAILED
    NAN_ENCOUNTERED = _lib.NAN_ENCOUNTERED
    UNKNOWN_ERROR = _lib.RUNNING


@dataclasses.dataclass
class ConvergenceCriteria:
    max_steps: int = 1500
    rtol: float | None = None  # None: 1e-6 in float32, 1e-9 in float64
    atol: float = 0.0


@dataclasses.dataclass
class LineSearch:
    c: float = 1.0e-4
    max_steps: int = 8
    overstep: float = 1.0


@dataclasses.dataclass
class LineSearchState:
    alpha: float
    f0: float
    f_alpha: float
    step: int
    ok: bool


@dataclasses.dataclass
class ConvergenceState:
    grad_norm: float
    grad_norm_first: float


@dataclasses.dataclass
class Solution:
    result: Result
    n_steps: int
    grad_norm: float
    grad_norm_first: float
    energy: float
    alpha: float
    beta: float
    line_search_steps: int
    line_search_ok: bool
    hess_diag_mean: float = 1.0  # the preconditioner's fill for zero diagonal entries

    @classmethod
    def from_stats(cls, st: _lib.PncgStats) -> Solution:
        return cls(Result(st.result), st.n_steps, st.grad_norm, st.grad_norm_first, st.energy, st.alpha, st.beta,
                   st.line_search_steps, bool(st.line_search_ok), st.hess_diag_mean)

    @property
    def success(self) -> bool:
        return self.result == Result.PRIMARY_SUCCESS

    @property
    def relative_grad_norm(self) -> float:
        return self.grad_norm / self.grad_norm_first if self.grad_norm_first else 0.0


@dataclasses.dataclass
class HessDampingState:
    """The fields the reference's progress logging reads from the optimizer
    state (exp/2026/05/06/toy/src/20-ext-force-stable-neo-hookean-collision.py:
    209,228-229).  This solver adds no damping to the Hessian, so ``factor``
    is 0; ``hess_diag_mean`` is the mean of the positive free diagonal
    entries, the preconditioner's fill for zero ones."""

    factor: float
    hess_diag_mean: float


@dataclasses.dataclass
class OptState:
    """Per-iteration view for step-by-step driving (init/step/terminate).
    ``direction`` is the last iteration's search direction over the free DOFs
    (the step taken was ``line_search_state.alpha * direction``; zero after
    init)."""

    n_steps: int
    line_search_state: LineSearchState
    convergence_state: ConvergenceState
    beta: float
    done: bool
    result: Result
    direction: torch.Tensor
    hess_damping_state: HessDampingState


@dataclasses.dataclass(frozen=True)
class CgSolution:
    result: Result
    n_iter: int
    residual: float
    residual_first: float

    @property
    def success(self) -> bool:
        return self.result == Result.PRIMARY_SUCCESS


class DeviceSolver:
    """One ``agb_solver`` bound to a device model."""

    def __init__(self, warp_model, params: _lib.PncgParams):
        self.warp_model = warp_model
        self.params = params
        h = ctypes.c_void_p()
        _lib.call("agb_solver_create", warp_model.handle, ctypes.byref(params), ctypes.byref(h))
        self.handle = h
        self._last_energy = float("nan")

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib.load().agb_solver_destroy(self.handle)
            self.handle = None

    def reset(self, u: torch.Tensor) -> None:
        u = u.to(self.warp_model.dtype).contiguous()
        _lib.call("agb_solver_reset", self.handle, ptr(u), stream_ptr(u.device))

    def iterate(self, n: int) -> None:
        _lib.call("agb_solver_iterate", self.handle, int(n), stream_ptr())

    def step(self) -> None:
        _lib.call("agb_solver_step", self.handle, stream_ptr())

    def save_state(self) -> torch.Tensor:
        """A checkpoint of the whole PNCG state (uint8 CPU tensor), for
        :meth:`load_state` on this or an identically built solver."""
        n = ctypes.c_size_t()
        _lib.call("agb_solver_checkpoint_size", self.handle, ctypes.byref(n))
        blob = torch.empty(n.value, dtype=torch.uint8)
        _lib.call("agb_solver_save", self.handle, ctypes.c_void_p(blob.data_ptr()), stream_ptr())
        return blob

    def load_state(self, blob: torch.Tensor) -> None:
        """Restore a checkpoint; the next iterate() continues from it.  A
        blob of the wrong length, or saved by a solver over another model or
        with other parameters, raises RuntimeError and changes nothing."""
        blob = blob.to(dtype=torch.uint8, device="cpu").contiguous()
        n = ctypes.c_size_t()
        _lib.call("agb_solver_checkpoint_size", self.handle, ctypes.byref(n))
        if blob.numel() != n.value:
            raise RuntimeError(f"checkpoint of {blob.numel()} bytes; this solver's checkpoints have {n.value}")
        _lib.call("agb_solver_load", self.handle, ctypes.c_void_p(blob.data_ptr()), ctypes.c_size_t(blob.numel()),
                  stream_ptr())

    def read_direction(self) -> torch.Tensor:
        """The last iteration's search direction p (full (n_points, 3), CPU
        tensor of the model dtype, zero on fixed DOFs and after reset)."""
        p = torch.empty((self.warp_model.n_points, 3), dtype=self.warp_model.dtype)
        _lib.call("agb_solver_read_direction", self.handle, ctypes.c_void_p(p.data_ptr()), stream_ptr())
        return p

    def read_gradient(self) -> tuple[torch.Tensor, torch.Tensor]:
        """The stored free gradient and clamped Hessian diagonal of the current
        iterate (full (n_points, 3) CPU tensors of the model dtype, zero on
        fixed DOFs)."""
        n, dt = self.warp_model.n_points, self.warp_model.dtype
        g = torch.empty((n, 3), dtype=dt)
        d = torch.empty((n, 3), dtype=dt)
        _lib.call("agb_solver_read_gradient", self.handle, ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                  stream_ptr())
        return g, d

    def read_reductions(self) -> dict:
        """The FP64 scalars of the last iteration's global reductions."""
        out = (ctypes.c_double * 5)()
        _lib.call("agb_solver_read_reductions", self.handle, out, stream_ptr())
        return {"hess_quad": out[0], "gd": out[1], "grad_norm": out[2], "precond_fill_inv": out[3], "beta": out[4]}

    def step_kernels(self) -> int:
        """Kernels one iteration launches (the nodes of the step graph)."""
        n = ctypes.c_int32()
        _lib.call("agb_solver_step_kernels", self.handle, ctypes.byref(n))
        return n.value

    def read(self, u_out: torch.Tensor | None = None) -> Solution:
        st = _lib.PncgStats()
        _lib.call("agb_solver_read", self.handle, ptr(u_out), ctypes.byref(st), stream_ptr())
        return Solution.from_stats(st)

    def adjoint(self, rhs: torch.Tensor, *, rtol: float = 1e-6, atol: float = 0.0,
                max_iter: int = 10000) -> tuple[torch.Tensor, "CgSolution"]:
        """Solve H(u*) lam = rhs on the free DOFs at the solver's current state
        (``agb_solver_adjoint``); lam is 0 on fixed components."""
        rhs = rhs.to(self.warp_model.dtype).contiguous()
        lam = torch.empty_like(rhs)
        prm = _lib.CgParams(int(max_iter), float(rtol), float(atol))
        st = _lib.CgStats()
        _lib.call("agb_solver_adjoint", self.handle, ptr(rhs), ptr(lam), ctypes.byref(prm), ctypes.byref(st),
                  stream_ptr(rhs.device))
        return lam, CgSolution(Result(st.result), st.n_iter, st.residual, st.residual_first)

    def minimize_host(self, u_host: torch.Tensor) -> Solution:
        """Solve from a HOST (CPU) tensor, in place (``agb_pncg_minimize_host``)."""
        if u_host.is_cuda or not u_host.is_contiguous() or u_host.dtype != self.warp_model.dtype:
            raise TypeError("u_host must be a contiguous CPU tensor of the model dtype")
        st = _lib.PncgStats()
        _lib.call("agb_pncg_minimize_host", self.handle, ctypes.c_void_p(u_host.data_ptr()), ctypes.byref(st),
                  stream_ptr())
        return Solution.from_stats(st)


class PNCG:
    def __init__(self, criteria: ConvergenceCriteria | None = None, line_search: LineSearch | None = None,
                 *, beta_max: float = 10.0, refresh_ratio: float = -1.0):
        self.criteria = criteria or ConvergenceCriteria()
        self.line_search = line_search or LineSearch()
        self.beta_max = beta_max
        # FP32 stable Neo-Hookean reference-state correction: refresh the FP64
        # reference gradient each time ||g|| drops by this factor; 0: off;
        # < 0: on (0.1) when rtol < 1e-5 asks for more than FP32 forces resolve
        self.refresh_ratio = refresh_ratio

    def params(self, dtype) -> _lib.PncgParams:
        p = _lib.PncgParams()
        _lib.load().agb_pncg_default_params(ctypes.byref(p))
        p.max_steps = int(self.criteria.max_steps)
        rtol = self.criteria.rtol
        if rtol is None:
            rtol = 1e-9 if dtype == torch.float64 else 1e-6
        p.rtol = float(rtol)
        p.atol = float(self.criteria.atol)
        p.max_backtracking = int(self.line_search.max_steps)
        p.armijo_c = float(self.line_search.c)
        p.overstep = float(self.line_search.overstep)
        p.beta_max = float(self.beta_max)
        p.refresh_ratio = float(self.refresh_ratio)
        return p

    def solver(self, problem) -> DeviceSolver:
        model = getattr(problem, "model", None)
        wm = getattr(model, "warp_model", None)
        if wm is None or not hasattr(wm, "handle"):
            raise TypeError("PNCG runs on apple_gb300 models (ForwardProblem over a Model)")
        # one device solver per (model, optimizer): cached on the model and
        # keyed weakly by the optimizer, so it is freed with either of them
        cache = wm.__dict__.setdefault("_pncg_solvers", weakref.WeakKeyDictionary())
        sv = cache.get(self)
        if sv is None:
            sv = cache[self] = DeviceSolver(wm, self.params(wm.dtype))
        return sv

    # -- Optimizer.minimize (forward/_forward.py:52-56) ------------------------
    def minimize(self, problem, state, free: torch.Tensor):
        sv = self.solver(problem)
        u = problem.before_trial(state, free).u
        sv.reset(u)
        sv.iterate(self.criteria.max_steps)
        u_out = torch.empty_like(u)
        sol = sv.read(u_out)
        return sol, dataclasses.replace(state, u=u_out)

    # -- step-wise driving (init / step / terminate / postprocess) -------------
    def init(self, problem, state, free: torch.Tensor) -> OptState:
        sv = self.solver(problem)
        sv.reset(problem.before_trial(state, free).u)
        return self._opt_state(problem, sv)

    def step(self, problem, state, opt_state: OptState):
        sv = self.solver(problem)
        sv.iterate(1)
        u_out = torch.empty_like(state.u)
        sv.read(u_out)
        return dataclasses.replace(state, u=u_out), self._opt_state(problem, sv, opt_state)

    def terminate(self, problem, state, opt_state: OptState):
        return opt_state.done, opt_state.result

    def postprocess(self, problem, state, opt_state: OptState, result) -> Solution:
        return self.solver(problem).read()

    def _opt_state(self, problem, sv: DeviceSolver, prev: OptState | None = None) -> OptState:
        s = sv.read()
        f0 = prev.line_search_state.f_alpha if prev is not None else s.energy
        done = s.result != Result.UNKNOWN_ERROR
        dof_map = problem.model.dof_map
        direction = dof_map.to_free(sv.read_direction().to(dof_map.free_indices.device))
        return OptState(
            n_steps=s.n_steps,
            line_search_state=LineSearchState(s.alpha, f0, s.energy, s.line_search_steps, s.line_search_ok),
            convergence_state=ConvergenceState(s.grad_norm, s.grad_norm_first),
            beta=s.beta,
            done=done,
            result=s.result,
            direction=direction,
            hess_damping_state=HessDampingState(0.0, s.hess_diag_mean),
        )
