"""Batched quasi-static solves: many independent models, one set of launches
per PNCG iteration (``agb_batch_*``), plus the small autotuner that picks the
tile and vertex-chunk shapes.

The reference steps one ``Forward`` per model (forward/_forward.py:52-56),
and each of its PNCG iterations is several FFI calls.  Here every running
model advances by one iteration per graph launch. Each model keeps its own
beta, step and termination, so the batched result of a model is the one its
own ``Forward.step()`` gives.
"""

from __future__ import annotations

import ctypes
import dataclasses
import time

import numpy as np
import torch

from . import _lib
from .fem import ptr, stream_ptr
from .pncg import PNCG, Solution


class BatchedForward:
    """``models``: :class:`apple_gb300.model.Model` objects of one dtype and
    one material family: ARAP potentials, or stable Neo-Hookean and muscle
    potentials (with any muscle in the batch, every cell runs as a muscle
    cell, the plain ones with zero activation).
    ``solve()`` minimises every model's energy from its current state (zero
    free displacement, fixed values applied)."""

    def __init__(self, models, optimizer: PNCG | None = None, *, chunk_verts: int = 0):
        if not models:
            raise ValueError("no models")
        self.models = list(models)
        self.dtype = self.models[0].dtype
        if any(m.dtype != self.dtype for m in self.models):
            raise TypeError("models of one batch share a dtype")
        self.optimizer = optimizer or PNCG()
        self.chunk_verts = int(chunk_verts)
        params = self.optimizer.params(self.dtype)
        handles = (ctypes.c_void_p * len(self.models))(*[m.warp_model.handle.value for m in self.models])
        h = ctypes.c_void_p()
        _lib.call("agb_batch_create", len(self.models), ctypes.cast(handles, ctypes.c_void_p), ctypes.byref(params),
                  self.chunk_verts, ctypes.byref(h))
        self.handle = h
        self.n_points = [m.n_points for m in self.models]
        self.offsets = np.concatenate([[0], np.cumsum(self.n_points)]).astype(np.int64)

    def __del__(self):
        if getattr(self, "handle", None) and _lib._lib is not None:
            _lib.load().agb_batch_destroy(self.handle)
            self.handle = None

    def info(self) -> tuple[int, int]:
        npt, nc = ctypes.c_int32(), ctypes.c_int32()
        _lib.call("agb_batch_info", self.handle, ctypes.byref(npt), ctypes.byref(nc))
        return npt.value, nc.value

    def initial_u(self, device="cuda") -> torch.Tensor:
        parts = [m.init().u.to(device) for m in self.models]
        return torch.cat(parts, 0).contiguous()

    def reset(self, u: torch.Tensor | None = None) -> None:
        u = self.initial_u() if u is None else u
        u = u.to(self.dtype).contiguous()
        self._u_device = u.device
        _lib.call("agb_batch_reset", self.handle, ptr(u), stream_ptr(u.device))

    def iterate(self, n: int) -> None:
        _lib.call("agb_batch_iterate", self.handle, int(n), stream_ptr())

    def step(self) -> None:
        _lib.call("agb_batch_step", self.handle, stream_ptr())

    def read(self, with_u: bool = True) -> tuple[list[Solution], list[torch.Tensor] | None]:
        n = len(self.models)
        st = (_lib.PncgStats * n)()
        u = None
        if with_u:
            u = torch.empty((int(self.offsets[-1]), 3), dtype=self.dtype, device="cuda")
        _lib.call("agb_batch_read", self.handle, ptr(u), ctypes.cast(st, ctypes.c_void_p), stream_ptr())
        sols = [Solution.from_stats(s) for s in st]
        us = None if u is None else [u[self.offsets[k]:self.offsets[k + 1]] for k in range(n)]
        return sols, us

    def solve(self, max_steps: int | None = None):
        """Reset every model and iterate until all have terminated."""
        self.reset()
        self.iterate(self.optimizer.criteria.max_steps if max_steps is None else max_steps)
        return self.read()


@dataclasses.dataclass
class TuneResult:
    tile_elems: int
    chunk_verts: int
    ms_per_iter: float
    table: list


def autotune(build_models, *, tile_elems=(256, 512, 1024), chunk_verts=(256, 512, 1024), iters: int = 10,
             optimizer: PNCG | None = None) -> TuneResult:
    """Pick the tile size (elements per tile, through the potentials'
    ``tile_elems``) and the vertex-pass chunk of the batched solver by timing
    ``iters`` iterations of each candidate on ``build_models(tile_elems)``
    (a list of models; a representative subset of the batch is enough)."""
    table = []
    best = None
    for te in tile_elems:
        models = build_models(te)
        for cv in chunk_verts:
            bf = BatchedForward(models, optimizer, chunk_verts=cv)
            bf.reset()
            bf.step()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(iters):
                bf.step()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / iters
            table.append((te, cv, ms))
            if best is None or ms < best[2]:
                best = (te, cv, ms)
            del bf
    return TuneResult(best[0], best[1], best[2], table)


def timed(fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0
