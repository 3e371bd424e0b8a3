"""Lifetimes of the device copies of a potential, on the host (no GPU: the C
library is replaced by a recorder).  A potential keeps one device copy per
vertex space, reuses it while that space lives, and destroys it when the
space goes -- a new space never receives a copy made for an earlier one,
even when Python reuses the earlier space's id."""

import ctypes
import gc

import numpy as np
import pytest

from apple_gb300 import _lib, fem, meshgen


class _Recorder:
    def __init__(self):
        self.next = 1000
        self.live = {}  # handle value -> kind
        self.calls = []

    def _new(self, kind):
        self.next += 8
        self.live[self.next] = kind
        return self.next

    def call(self, name, *args):
        self.calls.append((name, args))
        if name in ("agb_space_create", "agb_fem_create", "agb_model_create"):
            args[-1]._obj.value = self._new(name.split("_")[1])
        return 0

    def _destroy(self, kind):
        def destroy(h):
            v = h.value if isinstance(h, ctypes.c_void_p) else h
            assert self.live.pop(v) == kind, (kind, v)
            return 0
        return destroy

    def __getattr__(self, name):
        if name == "agb_fem_destroy":
            return self._destroy("fem")
        if name == "agb_space_destroy":
            return self._destroy("space")
        if name == "agb_model_destroy":
            return self._destroy("model")
        raise AttributeError(name)


@pytest.fixture
def rec(monkeypatch):
    gc.collect()  # earlier tests' handles go to the real library first
    r = _Recorder()
    monkeypatch.setattr(_lib, "call", r.call)
    monkeypatch.setattr(_lib, "load", lambda: r)
    monkeypatch.setattr(_lib, "_lib", r)
    return r


def _pot(cls=fem.StableNeoHookean):
    m = meshgen.grid(2, 2, 2)
    return cls(m.cells, 1.0, 10.0, points=m.points), m


def test_one_copy_per_space_destroyed_with_the_space(rec):
    pot, m = _pot()
    s1 = fem.Space(m.n_points, m.points)
    h1 = pot.on_space(s1)
    assert pot.on_space(s1).value == h1.value
    s2 = fem.Space(m.n_points, m.points)
    h2 = pot.on_space(s2)
    assert h2.value != h1.value
    v1 = h1.value
    del s1
    gc.collect()
    assert v1 not in rec.live and h2.value in rec.live
    del pot
    gc.collect()
    assert h2.value not in rec.live  # the potential takes its copies with it
    del s2
    gc.collect()
    assert not rec.live


def test_a_new_space_never_gets_an_earlier_copy(rec):
    pot, m = _pot()
    seen = set()
    ids = set()
    for _ in range(50):
        s = fem.Space(m.n_points, m.points)
        ids.add(id(s))
        h = pot.on_space(s).value
        assert h not in seen
        seen.add(h)
        del s
    assert len(seen) == 50
    gc.collect()
    assert sum(1 for k in rec.live.values() if k == "fem") == 0


def test_set_activation_reaches_every_live_copy(rec):
    pot, m = _pot(fem.StableNeoHookeanMuscle)
    s1, s2 = fem.Space(m.n_points, m.points), fem.Space(m.n_points, m.points)
    hs = {pot.on_space(s1).value, pot.on_space(s2).value, pot._standalone().value}
    rec.calls.clear()
    pot.set_activation(np.full((m.n_cells, 6), 0.01))
    got = {a[0].value for name, a in rec.calls if name == "agb_fem_set_activation"}
    assert got == hs


def test_models_rebuilt_from_one_potential(rec):
    """Two models built in turn from one potential: each is created over a
    live device copy on its own space; the first copy goes with the first
    model."""
    from apple_gb300.model import WarpModel

    pot, m = _pot()

    def fems_of_last_model_create():
        name, args = [c for c in rec.calls if c[0] == "agb_model_create"][-1]
        n = args[2]
        return [args[3][k] for k in range(n)]

    wm1 = WarpModel({"e": pot}, m.n_points, m.points)
    (f1,) = fems_of_last_model_create()
    assert rec.live[f1] == "fem"
    del wm1
    gc.collect()
    assert f1 not in rec.live and not any(k == "model" for k in rec.live.values())
    wm2 = WarpModel({"e": pot}, m.n_points, m.points)
    (f2,) = fems_of_last_model_create()
    assert rec.live[f2] == "fem" and f2 != f1
    del wm2
    gc.collect()
    assert not rec.live
