"""The optimizer's device-solver cache on the host (no GPU; the device solver
is replaced by a stand-in): one solver per (model, optimizer), reused across
calls, and released with either of them, so that an optimizer reused over
many models holds no solver of a model that is gone."""

import gc
import weakref

import torch

from apple_gb300 import pncg


class _WarpModel:
    handle = object()
    dtype = torch.float32


class _Model:
    def __init__(self, wm):
        self.warp_model = wm


class _Problem:
    def __init__(self, model):
        self.model = model


def _fake_solvers(monkeypatch):
    gc.collect()  # earlier tests' solvers go before the stand-in takes over
    made = []

    class FakeSolver:
        def __init__(self, warp_model, params):
            self.warp_model = warp_model
            self.params = params
            made.append(weakref.ref(self))

    monkeypatch.setattr(pncg, "DeviceSolver", FakeSolver)
    return made


def test_one_solver_per_model_and_optimizer(monkeypatch):
    made = _fake_solvers(monkeypatch)
    wm_a, wm_b = _WarpModel(), _WarpModel()
    pa, pb = _Problem(_Model(wm_a)), _Problem(_Model(wm_b))
    opt1 = pncg.PNCG(pncg.ConvergenceCriteria(max_steps=7))
    opt2 = pncg.PNCG()
    s1a = opt1.solver(pa)
    assert opt1.solver(pa) is s1a and opt1.solver(_Problem(_Model(wm_a))) is s1a
    assert s1a.params.max_steps == 7
    s1b, s2a = opt1.solver(pb), opt2.solver(pa)
    assert len({id(s1a), id(s1b), id(s2a)}) == 3 and len(made) == 3
    # the optimizer goes: its solvers go with it
    del opt2, s2a
    gc.collect()
    assert made[2]() is None
    assert opt1.solver(pa) is s1a


def test_solver_released_with_its_model(monkeypatch):
    made = _fake_solvers(monkeypatch)
    opt = pncg.PNCG()
    wm = _WarpModel()
    sv = opt.solver(_Problem(_Model(wm)))
    assert made[0]() is sv
    del sv, wm
    gc.collect()
    assert made[0]() is None  # the optimizer alone keeps nothing alive
