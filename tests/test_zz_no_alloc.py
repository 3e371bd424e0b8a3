"""The allocation-free energy entry point (agb_fem_fun_noalloc) against the
regular one (agb_fem_fun), through the C ABI, on two calls in a row.

agb_fem_fun_noalloc serves callers that must not allocate device memory
themselves, for example an FFI handler running under XLA's allocator, which
reserves most of the device up front: its per-call scratch is one file-scope
device array shared by all calls.  Two consecutive calls check that the
shared array's leftover contents (partials, completion counter) from the
previous call do not leak into the next result.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import _lib, meshgen

pytestmark = pytest.mark.gpu

TOL = {torch.float32: 1e-5, torch.float64: 1e-9}


def _potential(cls, dtype):
    m = meshgen.grid(12, 10, 14)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    pot = cls.from_pyvista(mesh, dtype=dtype)
    rng = np.random.default_rng(5)
    X = m.points - m.points.mean(0)
    u = X @ (0.05 * rng.normal(size=(3, 3))).T + 0.001 * np.sin(X @ rng.normal(size=(3, 3)))
    return pot, u


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("cls", [ag.StableNeoHookean, ag.Arap])
def test_fun_noalloc_matches_fun_twice(cls, dtype, cuda_device):
    pot, u = _potential(cls, dtype)
    U = torch.tensor(u, dtype=dtype, device=cuda_device)
    handle = pot._standalone()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    ref = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    _lib.call("agb_fem_fun", handle, ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(ref.data_ptr()), stream)
    for call in range(2):
        out = torch.full((1,), 3.0, dtype=torch.float64, device=cuda_device)  # accumulates
        _lib.call("agb_fem_fun_noalloc", handle, ctypes.c_void_p(U.data_ptr()),
                  ctypes.c_void_p(out.data_ptr()), stream)
        torch.cuda.synchronize(cuda_device)
        got = out.item() - 3.0
        assert got == pytest.approx(ref.item(), rel=TOL[dtype]), f"call {call}"


def _call_noalloc(handle, U, out, stream):
    _lib.call("agb_fem_fun_noalloc", handle, ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(out.data_ptr()), stream)


def test_fun_noalloc_rejects_a_muscle(cuda_device):
    """The muscle's activation stream is not read by this entry point, so it
    refuses muscle potentials with a status instead of a wrong energy."""
    m = meshgen.grid(3, 3, 3)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mesh.cell_data["activation"] = np.zeros((m.n_cells, 6))
    pot = ag.StableNeoHookeanMuscle.from_pyvista(mesh)
    U = torch.zeros((m.n_points, 3), dtype=torch.float32, device=cuda_device)
    out = torch.zeros(1, dtype=torch.float64, device=cuda_device)
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    with pytest.raises(RuntimeError, match="muscle"):
        _call_noalloc(pot._standalone(), U, out, stream)
    torch.cuda.synchronize(cuda_device)
    assert out.item() == 0.0


def test_fun_noalloc_tile_limit(cuda_device):
    """One element per tile: 65,536 cells fill the scratch array exactly and
    match agb_fem_fun; one cell more is refused before any launch."""
    m = meshgen.grid(30, 30, 16)  # 72,000 cells
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    rng = np.random.default_rng(11)
    u = 0.01 * rng.normal(size=(m.n_points, 3))
    U = torch.tensor(u, dtype=torch.float32, device=cuda_device)
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    for n_cells, fits in ((65536, True), (65537, False)):
        mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells[:n_cells]), mu, lam)
        pot = ag.StableNeoHookean.from_pyvista(mesh, tile_elems=1)
        handle = pot._standalone()
        n_tiles = ctypes.c_int32()
        _lib.call("agb_fem_info", handle, ctypes.byref(n_tiles), None)
        assert n_tiles.value == n_cells
        out = torch.zeros(1, dtype=torch.float64, device=cuda_device)
        if fits:
            ref = torch.zeros(1, dtype=torch.float64, device=cuda_device)
            _lib.call("agb_fem_fun", handle, ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(ref.data_ptr()), stream)
            _call_noalloc(handle, U, out, stream)
            torch.cuda.synchronize(cuda_device)
            assert out.item() == pytest.approx(ref.item(), rel=TOL[torch.float32])
        else:
            with pytest.raises(RuntimeError, match="65536"):
                _call_noalloc(handle, U, out, stream)
            torch.cuda.synchronize(cuda_device)
            assert out.item() == 0.0
