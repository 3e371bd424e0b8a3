"""The FP32 solver's global sums against FP64 recomputations at the 1.5M-tet
headline size (GB300).

In the FP32 build every global sum of the PNCG iteration starts as a plain
FP32 sum over a thread's few elements or vertices, continues in float-float
(hi + lo) warp and block trees and ends in FP64 (GB300's FP64 rate is about
1/64 of FP32, so FP64 leaves would cost more than the pass they sit in).
These tests recompute each sum in FP64 from the solver's own stored FP32
state and bound the relative error of the device value:

* p^T H p of a direction at its base point (sets alpha_0): against the FP64 C
  restatement of the reference's hess_quad kernel at the same u and p (this
  sum's terms are FP32 element math, so its bar is the FP32 element bar);
* ||g|| and g . p_next = -g^T P g + beta p.g (the Dai-Kou update): against
  FP64 sums over the stored g, Hessian diagonal d and direction p;
* the total energy the solver reports: against the FP64 C restatement's fun.

The reference keeps these sums in FP64 (JAX_ENABLE_X64, jnp.vdot in the
PNCG proxy benches/bench_pncg_branching_backends.py:606-679).
"""

import numpy as np
import pytest
import torch

import apple_gb300 as ag
from apple_gb300 import meshgen
from oracle import build_c
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

NX, NY, NZ = 50, 50, 120
BOUND = 1e-6  # relative error of a pure reduction against its FP64 recomputation
ELEM = 1e-5  # the same for sums of FP32 element terms (the FP32 element-math bar)


@pytest.fixture(scope="module")
def headline(cuda_device):
    m = meshgen.grid(NX, NY, NZ, h=1.0 / NX)
    assert m.n_cells == 1_500_000
    lam, mu = meshgen.lame_converter(1e5, 0.49)
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    top = meshgen.face_mask(m, 2, "max")
    mask[top] = True
    fv[top, 2] = 0.3 * m.points[:, 2].max()
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b = ag.ModelBuilder(dtype=torch.float32)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh))
    model = b.finalize()
    dhdX, dV = O.region_compute_grad(m.points, m.cells)
    cm = build_c.CModel(1, m.cells, dhdX, dV, mu, lam, m.n_points, mask=mask.astype(np.uint8))
    u0 = torch.tensor(np.where(mask, fv, 0.0), dtype=torch.float32, device=cuda_device)
    return m, mask, model, cm, u0


@pytest.mark.parametrize("n_before", [1, 40, 400])
def test_reductions_match_fp64_recomputation(headline, n_before, cuda_device):
    m, mask, model, cm, u0 = headline
    free = ~mask
    sv = ag.PNCG(ag.ConvergenceCriteria(max_steps=10**6, rtol=0.0)).solver(ag.ForwardProblem(model))
    sv.reset(u0)
    sv.iterate(n_before)
    u_j = torch.empty_like(u0)
    sv.read(u_j)
    sv.iterate(1)  # iteration j: direction p_j and p_j^T H p_j at x_j
    u_next = torch.empty_like(u0)
    stats = sv.read(u_next)
    red = sv.read_reductions()
    p = sv.read_direction().double().numpy()
    g, d = (t.double().numpy() for t in sv.read_gradient())

    # p^T H p at the direction's base point (the direction pass reads the hi
    # word of x; u_j is hi + lo rounded once, within an ulp of it)
    hq64 = cm.eval(u_j.double().cpu().numpy(), p, flags=16)["hess_quad"]
    assert abs(red["hess_quad"] - hq64) <= ELEM * abs(hq64)

    gf, df, pf = g[free], d[free], p[free]
    gn64 = float(np.sqrt(np.sum(gf * gf)))
    assert abs(red["grad_norm"] - gn64) <= BOUND * gn64
    assert abs(stats.grad_norm - gn64) <= BOUND * gn64

    # -g^T P g + beta p.g with P = 1/|d| (the fill 1/mean for zero entries)
    ad = np.abs(df)
    P = np.where(ad > 0, 1.0 / np.where(ad > 0, ad, 1.0), red["precond_fill_inv"])
    gpg = float(np.sum(gf * gf * P))
    pg = float(np.sum(pf * gf))
    gd64 = -gpg + red["beta"] * pg
    scale = gpg + abs(red["beta"] * pg)
    assert abs(red["gd"] - gd64) <= BOUND * scale
    fill64 = float(np.count_nonzero(ad > 0) / np.sum(ad))
    assert abs(red["precond_fill_inv"] - fill64) <= BOUND * fill64

    # total energy at the iterate (the solver's on-demand energy pass)
    e64 = cm.eval(u_next.double().cpu().numpy(), None, flags=1)["fun"]
    assert abs(stats.energy - e64) <= ELEM * abs(e64)
