"""The tile / warp-group plan on the host (``agb_plan_tiles``, no GPU): every
cell lands in exactly one tile and one warp group with its corner set kept;
tiles respect their element and vertex limits; in every
group and corner slot the vertices are distinct (the colouring that lets a
warp accumulate in shared memory without atomics or lost updates); and the
plan is deterministic."""

import ctypes

import numpy as np
import pytest

from apple_gb300 import _lib, meshgen


def _plan(m, tile_elems=0):
    lib = _lib.load()
    nc = m.n_cells
    cells = np.ascontiguousarray(m.cells, np.int32)
    pts = np.ascontiguousarray(m.points, np.float64)
    tile = np.empty(nc, np.int32)
    group = np.empty(nc, np.int32)
    slots = np.empty((nc, 4), np.int32)
    nt, ng = ctypes.c_int32(), ctypes.c_int32()
    _lib.call("agb_plan_tiles", m.n_points, nc, cells.ctypes.data, pts.ctypes.data, tile_elems, ctypes.byref(nt),
              ctypes.byref(ng), tile.ctypes.data, group.ctypes.data, slots.ctypes.data)
    del lib
    return nt.value, ng.value, tile, group, slots


@pytest.mark.parametrize("kind,tile_elems", [("grid", 0), ("grid", 100), ("ball", 0), ("ball", 37)])
def test_plan_invariants(kind, tile_elems):
    m = meshgen.grid(9, 8, 10) if kind == "grid" else meshgen.ball(3000, 600, seed=1)
    nt, ng, tile, group, slots = _plan(m, tile_elems)
    cap = tile_elems or 1024
    # every cell once with its corner set (the colouring permutes corners; the
    # element gradients are permuted alike, so the order's orientation is free)
    np.testing.assert_array_equal(np.sort(slots, axis=1), np.sort(m.cells, axis=1))
    assert tile.min() >= 0 and tile.max() == nt - 1
    assert group.min() >= 0 and group.max() == ng - 1
    for t in range(nt):
        sel = tile == t
        assert 0 < sel.sum() <= cap
        assert np.unique(slots[sel]).size <= 256
    for g in range(ng):
        sel = group == g
        assert 0 < sel.sum() <= 32
        assert np.unique(tile[sel]).size == 1  # a group never spans tiles
        for a in range(4):
            assert np.unique(slots[sel, a]).size == sel.sum(), (g, a)  # distinct per corner slot


def test_plan_is_deterministic_and_groups_are_full():
    m = meshgen.ball(3000, 600, seed=2)
    a = _plan(m)
    b = _plan(m)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    nt, ng, tile, group, slots = a
    fill = np.bincount(group) / 32.0
    assert fill.mean() > 0.8  # warp lanes mostly busy


def test_plan_rejects_bad_connectivity():
    m = meshgen.grid(2, 2, 2)
    bad = m.cells.copy()
    bad[0, 0] = m.n_points
    with pytest.raises(RuntimeError):
        _plan(meshgen.TetMesh(m.points, bad))


def test_plan_of_no_cells_is_empty():
    m = meshgen.grid(2, 2, 2)
    nt, ng, tile, group, slots = _plan(meshgen.TetMesh(m.points, np.zeros((0, 4), np.int32)))
    assert nt == 0 and ng == 0 and tile.size == 0
