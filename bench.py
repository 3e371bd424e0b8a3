#!/usr/bin/env python
"""PNCG iterations/s on the 1.5M-tet stable Neo-Hookean grid (GB300).

Workload: 50 x 50 x 120 cubes of side 1/50 split 5 tets per cube
(1,500,000 tets, 314,721 vertices), E = 1e5, nu = 0.49, z = 0 face fixed,
z = max face displaced +30% of the length along z, FP32 element arithmetic
with float-float/FP64 reductions.  A step is one PNCG iteration (direction
pass, gradient pass, vertex pass, and the two reference-state refresh passes
that return at once unless a refresh is due: one CUDA graph launch); the PNCG
state carries across steps.  L2 is flushed (256 MiB device write) before every
timed step; each step is timed with CUDA events on the launching stream.

Also reported: the dominant pass timed alone against the measured HBM peak
(roofline), the end-to-end rate through the public host-buffer API
(``minimize_host``: copy u in, solve a fixed number of iterations, copy u
out), and the CPU baseline (the C/OpenMP FP64 restatement of the reference
path on this host's cores).

``--impl reference`` times that CPU restatement on the same workload.
Multi-GPU (torchrun): independent replicas, one per rank (weak scaling).

Other workloads (``--config``): ``grid64`` (64x64x96 cells, ARAP and stable
Neo-Hookean, FP32 and FP64), ``irregular`` (Delaunay ball), ``batched`` (512
uneven grids in one batch vs one by one), ``adjoint`` (138k-tet material
gradient vs finite differences), ``muscle`` (the headline grid as an activated
muscle) and ``hbm-sizes`` (cold bandwidth vs bytes per launch).
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NX, NY, NZ = 50, 50, 120
E_MOD, NU = 1e5, 0.49
STRETCH = 0.3
WORKLOAD = "snh_grid_50x50x120_1.5M_tets_stretch30"
METRIC = "PNCG iters/s at 1.5M tets (stable Neo-Hookean)"
# algorithmic bytes (per tet: 4 int32 ids + 9 fp32 Dm^-1 + dV + mu + lambda;
# per vertex per iteration: x, p_prev, g_prev read + x, p, g, diag written)
B_TET, B_VERT = 64, 84


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--e2e-iters", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU baseline work")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP32-vs-FP64 accuracy record")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and adjoint sub-records")
    ap.add_argument("--small", action="store_true", help="16x16x40 grid (smoke / profiling runs)")
    ap.add_argument("--config", choices=["plain", "adjoint", "batched", "grid64", "irregular", "irregular-study",
                                         "hbm-sizes", "muscle"],
                    default="plain",
                    help="plain: the headline PNCG line; adjoint: the 138k-tet adjoint workload; "
                         "batched: 512 uneven meshes in one batch vs solved one by one; grid64: the "
                         "64x64x96 grid (ARAP and stable Neo-Hookean, FP32 and FP64); irregular: the "
                         "Delaunay ball; hbm-sizes: cold-L2 read / copy bandwidth of plain torch kernels "
                         "vs transfer size (the achievable bandwidth of one pass of a given size); muscle: the "
                         "headline grid with an activation-prestrained stable Neo-Hookean muscle vs the plain material")
    ap.add_argument("--n-meshes", type=int, default=512, help="batched: number of meshes")
    ap.add_argument("--fd-cells", type=int, default=8,
                    help="adjoint: cells checked by central differences (half random, half largest |dL/dtheta|)")
    ap.add_argument("--profile", action="store_true",
                    help="run warmup iterations, then each pass `steps` times as plain launches (ncu captures)")
    return ap.parse_args()


def _mesh(small=False):
    from apple_gb300 import meshgen

    nx, ny, nz = (16, 16, 40) if small else (NX, NY, NZ)
    m = meshgen.grid(nx, ny, nz, h=1.0 / nx)
    lam, mu = meshgen.lame_converter(E_MOD, NU)
    import numpy as np

    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    top = meshgen.face_mask(m, 2, "max")
    mask[top] = True
    fv[top, 2] = STRETCH * m.points[:, 2].max()
    return m, float(mu), float(lam), mask, fv


def headline_config(small: bool, world: int) -> dict:
    """The workload description both arms print (the GPU arm and the CPU
    reference arm), so that their lines name the same configuration."""
    nx, ny, nz = (16, 16, 40) if small else (NX, NY, NZ)
    return {"workload": WORKLOAD if not small else "snh_grid_16x16x40", "n_tets": 5 * nx * ny * nz,
            "n_vertices": (nx + 1) * (ny + 1) * (nz + 1), "E": E_MOD, "nu": NU,
            "step": "one PNCG iteration",
            "l2": "GPU arm: flushed before every step (256 MiB write); CPU arm: no flush",
            "parallelism": f"replicas x{world}"}


def _measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        # one synchronous sample at the start, so that a timed region shorter
        # than the sampling period still has a record
        self.edges = self._sample_once()
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(gpu_index)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def _sample_once(self) -> list:
        try:
            r = subprocess.run(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                "-i", str(self.gpu)], capture_output=True, text=True, timeout=20)
        except (OSError, subprocess.TimeoutExpired):
            return []
        return [row.split(",") for row in r.stdout.strip().splitlines() if row.count(",") >= 8]

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.seek(0)
        during = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        self.edges += self._sample_once()  # and one at the end
        rows = during if during else self.edges
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        reasons = sorted({n for r in rows for n, v in zip(self.NAMES, r[5:9]) if v.strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "source": "sampled every 100 ms during the timed region" if during
                else "one sample at the start and one at the end (timed region shorter than the period)"}


def _dist():
    """(world, rank, local) from the torchrun environment; NCCL across GPUs, gloo without CUDA."""
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cuda = torch.cuda.is_available()
    if cuda:
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if cuda else "gloo")
    return world, rank, local


def _barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def _max_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _aggregate(world, units_per_rank: float, local_seconds: float):
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    total_s = _max_over_ranks(world, local_seconds)
    return world * units_per_rank / total_s, total_s


def cpu_reference(steps_req: int, budget: float, small: bool = False, warmup: int = 1) -> dict:
    """The C/OpenMP FP64 restatement of the reference path on this host:
    ``warmup`` untimed iterations (which also size the sample to ``budget``
    seconds), then up to ``steps_req`` timed iterations of a fresh solve."""
    import numpy as np

    from oracle import build_c
    from oracle import fem_oracle as O

    m, mu, lam, mask, fv = _mesh(small)
    dhdX, dV = O.region_compute_grad(m.points, m.cells)
    cm = build_c.CModel(1, m.cells, dhdX, dV, mu, lam, m.n_points, mask=mask.astype(np.uint8))
    u0 = np.where(mask, fv, 0.0)
    w = max(1, int(warmup))
    t0 = time.perf_counter()
    cm.pncg(u0, max_steps=w, rtol=0.0)
    t1 = (time.perf_counter() - t0) / w
    n = int(max(2, min(steps_req, budget / max(t1, 1e-6))))
    t0 = time.perf_counter()
    _, st = cm.pncg(u0, max_steps=n, rtol=0.0)
    dt = time.perf_counter() - t0
    return {"value": st.n_steps / dt, "unit": "iter/s", "cores": build_c.threads(), "kind": "port",
            "iters": int(st.n_steps), "seconds": dt, "warmup": w,
            "sample": f"{st.n_steps} PNCG iterations of the full {m.n_cells}-tet workload from its initial "
                      f"state (C/OpenMP FP64 restatement of the reference kernels; one pass per method, "
                      f"atomic scatter; plus one trailing evaluation)"}


def headline_accuracy(pot, model, m, mu, lam, mask, fv, u0, u32, dev, n_mid=100, rtol_tight=1e-8,
                      rtol64=1e-10) -> dict:
    """FP32 against FP64 on the headline workload, outside the timed region.

    * energy and free gradient against the FP64 C restatement of the
      reference kernels: of the FP32 API path (``fun`` / ``grad`` of the FP32
      potential) at the initial state and at the FP32 solver's iterate after
      ``n_mid`` iterations, and of the solver's own stored gradient (the
      reference-state correction) at that iterate;
    * how converged the headline's FP32 answer u32 (rtol 1e-6) is in FP64:
      |g64(u32)| / |g64(u0)| on the free DOFs;
    * displacements against the FP64 build's solve to ``rtol64`` (the FP64
      kernels are pinned to the oracle at 1e-9): the FP32 solve to
      ``rtol_tight`` (FP32 arithmetic at matched, tight tolerance), and u32
      (which adds the tolerance's own error: at nu = 0.49 and 30% stretch
      the equilibrium is ill-conditioned, so ||g||/||g0|| = 1e-6 leaves a
      displacement error of order 1% of the diagonal in any precision).
    """
    import numpy as np
    import torch

    import apple_gb300 as ag
    from oracle import build_c
    from oracle import fem_oracle as O

    dhdX, dV = O.region_compute_grad(m.points, m.cells)
    cm = build_c.CModel(1, m.cells, dhdX, dV, mu, lam, m.n_points, mask=mask.astype(np.uint8))
    free = ~mask

    def c64(u):
        r = cm.eval(np.asarray(u, np.float64), None, flags=3)
        return r["fun"], r["grad"][free]

    def gpu32(u):
        U = torch.as_tensor(np.asarray(u, np.float32), device=dev)
        e = torch.zeros(1, dtype=torch.float64, device=dev)
        g = torch.zeros_like(U)
        pot.fun(U, e)
        pot.grad(U, g)
        torch.cuda.synchronize(dev)
        return float(e.item()), g.double().cpu().numpy()[free]

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))

    u0h = u0.double().cpu().numpy()
    e64_0, g64_0 = c64(u0h)
    e32_0, g32_0 = gpu32(u0h)
    sv = ag.PNCG(ag.ConvergenceCriteria(max_steps=n_mid, rtol=0.0)).solver(ag.ForwardProblem(model))
    sv.reset(u0)
    sv.iterate(n_mid)
    u_mid = torch.empty_like(u0)
    sv.read(u_mid)
    gs, _ = sv.read_gradient()
    um = u_mid.double().cpu().numpy()
    e64m, g64m = c64(um)
    e32m, g32m = gpu32(um)
    uc = u32.double().cpu().numpy()
    e64c, g64c = c64(uc)
    e32c, _ = gpu32(uc)
    tight = ag.PNCG(ag.ConvergenceCriteria(max_steps=40000, rtol=rtol_tight)).solver(ag.ForwardProblem(model))
    tight.reset(u0)
    tight.iterate(40000)
    ut = torch.empty_like(u0)
    st_t = tight.read(ut)
    t0 = time.perf_counter()
    sol64, u64 = _solve_f64(m, mu, lam, mask, fv, rtol64, dev)
    t64 = time.perf_counter() - t0
    u64h = u64.cpu().numpy()
    diag = float(np.linalg.norm(m.points.max(0) - m.points.min(0)))
    # two equilibria or one?  each precision restarted from the other's answer
    uth = ut.double().cpu().numpy()
    sol64b, u64b = _solve_f64(m, mu, lam, mask, fv, rtol64, dev, u_init=ut.double())
    back = ag.PNCG(ag.ConvergenceCriteria(max_steps=40000, rtol=rtol_tight)).solver(ag.ForwardProblem(model))
    back.reset(u64.float())
    back.iterate(40000)
    u32b = torch.empty_like(u0)
    back.read(u32b)
    e_t, _ = c64(uth)
    e_64, g_64 = c64(u64h)
    e_64b, _ = c64(u64b.cpu().numpy())
    restarts = {
        "fp64_energy": {f"at_f32_rtol_{rtol_tight:g}": e_t, "at_fp64": e_64, "at_fp64_from_f32": e_64b},
        "fp64_from_f32_answer": {"iters": sol64b.n_steps, "rel_grad": sol64b.grad_norm / sol64b.grad_norm_first,
                                 "moved_over_diag": float(np.abs(u64b.cpu().numpy() - uth).max()) / diag,
                                 "to_fp64_answer_over_diag": float(np.abs(u64b.cpu().numpy() - u64h).max()) / diag},
        "f32_from_fp64_answer_over_diag": float(np.abs(u32b.double().cpu().numpy() - u64h).max()) / diag,
        "rel_diff_over_diag_quantiles_f32_vs_fp64": np.quantile(np.abs(uth - u64h).max(axis=1) / diag,
                                                                  [0.5, 0.9, 0.99, 1.0]).tolist(),
    }
    return {
        "reference": "FP64 C restatement of the reference kernels (energy, gradient); the FP64 build's PNCG "
                     f"to rtol {rtol64:g} (displacement)",
        "energy_rel": {"u0": abs(e32_0 - e64_0) / abs(e64_0), f"iterate_{n_mid}": abs(e32m - e64m) / abs(e64m),
                       "u32": abs(e32c - e64c) / abs(e64c)},
        "grad_rel_l2": {"u0_api": rel(g32_0, g64_0), f"iterate_{n_mid}_api": rel(g32m, g64m),
                        f"iterate_{n_mid}_solver": rel(gs.double().numpy()[free], g64m)},
        "fp64_rel_grad_of_u32": float(np.linalg.norm(g64c) / np.linalg.norm(g64_0)),
        "disp_err_over_diag": {f"f32_rtol_{rtol_tight:g}": float(np.abs(ut.double().cpu().numpy() - u64h).max()) / diag,
                               "u32_rtol_1e-06": float(np.abs(uc - u64h).max()) / diag},
        "restarts": restarts,
        "f32_tight_solve": {"result": st_t.result.name, "iters": st_t.n_steps,
                            "rel_grad": st_t.grad_norm / st_t.grad_norm_first},
        "fp64_solve": {"result": sol64.result.name, "iters": sol64.n_steps, "seconds": t64,
                       "rel_grad": sol64.grad_norm / sol64.grad_norm_first},
        "bars": {"energy_rel": 1e-5, "grad_rel_l2": 1e-5, "disp_err_over_diag": 1e-4},
    }


def _solve_f64(m, mu, lam, mask, fv, rtol, dev, max_steps=40000, u_init=None):
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen

    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b = ag.ModelBuilder(dtype=torch.float64)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=torch.float64))
    model = b.finalize()
    sv = ag.PNCG(ag.ConvergenceCriteria(max_steps=max_steps, rtol=rtol)).solver(ag.ForwardProblem(model))
    sv.reset(torch.tensor(np.where(mask, fv, 0.0), dtype=torch.float64, device=dev) if u_init is None else u_init)
    sv.iterate(max_steps)
    u = torch.empty((m.n_points, 3), dtype=torch.float64, device=dev)
    sol = sv.read(u)
    return sol, u


def loop_overhead_us(dev, n=2000) -> float:
    """Microseconds per iteration of agb_solver_iterate's device loop on a
    4x4x4-cell grid (320 tets), where the kernels have almost no work: the
    fixed cost of an iteration's launches and grid-wide completions."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen

    m = meshgen.grid(4, 4, 4)
    lam, mu = meshgen.lame_converter(E_MOD, NU)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((m.n_points, 3))
    b = ag.ModelBuilder(dtype=torch.float32)
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    b.add_potential(ag.StableNeoHookean.from_pyvista(mesh))
    fm = meshgen.TetMesh(m.points, m.cells)
    fm.point_data["Force"] = meshgen.lumped_gravity(m, 1000.0)
    fm.point_data["GlobalPointId"] = np.arange(m.n_points)
    b.add_potential(ag.ExternalForce.from_pyvista(fm))
    model = b.finalize()
    sv = ag.PNCG(ag.ConvergenceCriteria(max_steps=10**6, rtol=0.0)).solver(ag.ForwardProblem(model))
    u0 = torch.zeros((m.n_points, 3), dtype=torch.float32, device=dev)
    sv.reset(u0)
    sv.iterate(3)
    torch.cuda.synchronize(dev)
    sv.reset(u0)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    sv.iterate(n)
    st = sv.read()
    dt = time.perf_counter() - t0
    return 1e6 * dt / max(st.n_steps, 1)


def batched_record(n=64, dims=(4, 40), max_steps=2000, rtol=1e-6, n_check=3, seed=0) -> dict:
    """The batched form against the plain per-mesh form (a bounded sample of
    the 512-mesh workload, outside the timed region): ``n`` uneven grids of
    the batched workload's generator, each run to ``rtol`` or ``max_steps``
    both ways.  A mesh in the batch runs exactly the single-mesh iteration
    (its own beta, step and termination), so both forms reach the same
    accuracy; the record checks that (max |u_batch - u_plain| / diagonal) and
    measures both against FP64 solves of the C restatement of the reference
    path on the ``n_check`` smallest meshes.  The reference steps one
    ``Forward`` per model (forward/_forward.py:52-56)."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen
    from apple_gb300.batch import BatchedForward
    from oracle import build_c
    from oracle import fem_oracle as O

    rng = np.random.default_rng(seed)
    cases = [meshgen.batch_case(k, rng, dims=dims, h=1.0 / 400) for k in range(n)]
    crit = ag.ConvergenceCriteria(max_steps=max_steps, rtol=rtol)
    models = _batch_models(cases, torch.float32)
    bf = BatchedForward(models, ag.PNCG(crit))
    n_points, n_cells = bf.info()
    bf.solve(max_steps=3)  # graph capture
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bf.reset()
    bf.iterate(max_steps)
    sols, us = bf.read()
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    plain_u, plain_sols, t_plain = [], [], 0.0
    for mdl in models:
        opt = ag.PNCG(crit)
        fwd = ag.Forward(mdl, opt)
        opt.solver(fwd.problem)  # build and capture outside the timing, as for the batch
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        sol = fwd.step()
        torch.cuda.synchronize()
        t_plain += time.perf_counter() - t1
        plain_sols.append(sol)
        plain_u.append(fwd.state.u)
    diag = [float(np.linalg.norm(m.points.max(0) - m.points.min(0))) for m, _ in cases]
    d_bp = max(float((u.double() - v.double()).abs().max()) / d for u, v, d in zip(us, plain_u, diag))
    err_b, err_p = [], []
    for k in sorted(range(n), key=lambda k: cases[k][0].n_cells)[:n_check]:
        m, f = cases[k]
        dhdX, dV = O.region_compute_grad(m.points, m.cells)
        cm = build_c.CModel(1, m.cells, dhdX, dV, m.cell_data["mu"], m.cell_data["lambda"], m.n_points,
                            mask=np.asarray(m.point_data["FixedMask"], np.uint8), force=f)
        u_ref, _ = cm.pncg(np.zeros((m.n_points, 3)), max_steps=50000, rtol=1e-10)
        err_b.append(float(np.abs(us[k].double().cpu().numpy() - u_ref).max()) / diag[k])
        err_p.append(float(np.abs(plain_u[k].double().cpu().numpy() - u_ref).max()) / diag[k])
    iters = [s.n_steps for s in sols]
    # the device loop's fixed cost per iteration (five kernels in a graph
    # WHILE node): the same loop over two 4x4x4-cell grids, where the kernels
    # have almost no work; a persistent kernel with grid barriers between the
    # phases could save at most this much per iteration
    tiny = [meshgen.batch_case(k, np.random.default_rng(99), dims=(4, 4), h=1.0 / 400) for k in range(2)]
    tb = BatchedForward(_batch_models(tiny, torch.float32),
                        ag.PNCG(ag.ConvergenceCriteria(max_steps=10**6, rtol=0.0)))
    tb.solve(max_steps=3)
    torch.cuda.synchronize()
    tb.reset()
    t0 = time.perf_counter()
    tb.iterate(2000)
    tsols, _ = tb.read(with_u=False)
    torch.cuda.synchronize()
    t_tiny = time.perf_counter() - t0
    return {
        "workload": f"{n} grids of the batched workload's generator, {dims[0]}-{dims[1]} cells per axis "
                    f"(seed {seed}), FP32, rtol {rtol:g} or {max_steps} iterations",
        "n_meshes": n, "n_tets": n_cells, "n_vertices": n_points,
        "batched_s": t_batch, "plain_s": t_plain, "speedup": t_plain / t_batch,
        "iters_total": int(sum(iters)), "iters_equal": all(s.n_steps == p.n_steps for s, p in zip(sols, plain_sols)),
        "converged": {"batched": int(sum(s.result == ag.Result.PRIMARY_SUCCESS for s in sols)),
                      "plain": int(sum(s.result == ag.Result.PRIMARY_SUCCESS for s in plain_sols))},
        "max_diff_batched_vs_plain_over_diag": d_bp,
        "fp64_reference_err_over_diag": {"meshes": n_check, "batched": max(err_b), "plain": max(err_p),
                                         "reference": "FP64 C restatement of the reference PNCG, rtol 1e-10"},
        "loop_us_per_iter": {"this_batch": 1e6 * t_batch / max(iters),
                             "two_4x4x4_grids": 1e6 * t_tiny / max(max(s.n_steps for s in tsols), 1)},
    }


def adjoint_record(small=False, seed=0) -> dict:
    """The adjoint form against the plain forward (the 24x24x48-cell adjoint
    workload, 138,240 tets, one theta per tet scaling mu; outside the timed
    region): one forward solve (FP32, rtol 1e-7) plus the device adjoint (CG
    with H p, then the material VJP) gives all 138,240 derivatives, where
    the plain form needs two forward solves per parameter.  Accuracy: the
    directional derivative along a random direction against central
    differences of two FP64 forwards (started from u*, stopped at 1e-12 of
    the cold-start gradient), and FP32 vs FP64 adjoint.  The reference's
    recipe: exp/2025/09/24/inverse-grin/src/32-inverse.py:223-260."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen
    from apple_gb300.adjoint import MaterialEquilibrium

    rng = np.random.default_rng(seed)
    nx, ny, nz = (6, 6, 12) if small else (24, 24, 48)
    m = meshgen.grid(nx, ny, nz, h=1.0 / nx)
    lam0, mu0 = meshgen.lame_converter(E_MOD, NU)
    theta = rng.uniform(0.5, 2.0, m.n_cells)
    theta_star = rng.uniform(0.5, 2.0, m.n_cells)
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    top = meshgen.face_mask(m, 2, "max")
    mask[top] = True
    fv[top, 2] = STRETCH * m.points[:, 2].max()
    surf = np.zeros(m.n_points, bool)
    for ax in range(3):
        for side in ("min", "max"):
            surf |= meshgen.face_mask(m, ax, side)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    lam = lam0 * np.ones(m.n_cells)
    p32 = MaterialEquilibrium(mesh, ag.StableNeoHookean, dtype=torch.float32,
                              criteria=ag.ConvergenceCriteria(max_steps=200000, rtol=1e-7), cg_rtol=1e-6)
    p64 = MaterialEquilibrium(mesh, ag.StableNeoHookean, dtype=torch.float64,
                              criteria=ag.ConvergenceCriteria(max_steps=200000, rtol=1e-10), cg_rtol=1e-10)
    dev = torch.device("cuda")
    si = torch.tensor(np.flatnonzero(surf), device=dev)
    target = p64.solve(mu0 * theta_star, lam)[si].clone()

    def loss(u):
        return 0.5 * float(((u.double()[si] - target) ** 2).sum())

    def gradient(prob, th):
        u = prob.solve(mu0 * th, lam)
        g = torch.zeros_like(u)
        g[si] = (u.double()[si] - target).to(u.dtype)
        d = prob.vjp(g)["mu"].double().cpu().numpy() * mu0
        return loss(u), d, dict(prob.timings), prob.stats

    gradient(p32, theta)  # warm-up: graph capture, kernel attributes
    _, d32, t32, s32 = gradient(p32, theta)
    _, d64, _, s64 = gradient(p64, theta)
    g_first = s64.forward.grad_norm_first
    p_fd = MaterialEquilibrium(mesh, ag.StableNeoHookean, dtype=torch.float64,
                               criteria=ag.ConvergenceCriteria(max_steps=400000, rtol=0.0, atol=1e-12 * g_first))
    u_base = p_fd.solve(mu0 * theta, lam, u0=p64.solve(mu0 * theta, lam)).clone()
    v = rng.normal(size=m.n_cells)
    hd = 1e-2
    lp = loss(p_fd.solve(mu0 * theta * (1.0 + hd * v), lam, u0=u_base))
    lm = loss(p_fd.solve(mu0 * theta * (1.0 - hd * v), lam, u0=u_base))
    fd_dir = (lp - lm) / (2 * hd)
    dir32, dir64 = float(np.dot(d32, v * theta)), float(np.dot(d64, v * theta))
    fwd32, adj32 = t32["forward"], t32["adjoint"]
    return {
        "workload": ADJ_WORKLOAD if not small else "snh_grid_6x6x12_adjoint",
        "n_tets": m.n_cells, "n_params": m.n_cells,
        "forward_s": fwd32, "forward_iters": s32.forward.n_steps, "adjoint_s": adj32, "cg_iters": s32.cg.n_iter,
        "gradient_s": fwd32 + adj32,
        "plain_s_est": 2 * m.n_cells * fwd32,
        "plain": "central differences of the plain forward: 2 solves per parameter",
        "speedup_est": 2 * m.n_cells * fwd32 / (fwd32 + adj32),
        "adjoint_over_one_forward": adj32 / fwd32,
        "directional_rel_err_vs_fd": {"f32": abs(dir32 - fd_dir) / abs(fd_dir),
                                      "f64": abs(dir64 - fd_dir) / abs(fd_dir)},
        "f32_vs_f64_adjoint_rel": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64)),
    }


def run_reference(a) -> None:
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and rank != 0:
        return
    r = cpu_reference(a.steps, max(a.cpu_budget * 3, 30.0), a.small, a.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": "iter/s", "n_gpus": a.gpus,
        "steps": r["iters"], "warmup": r["warmup"], "ms_per_step": 1e3 / r["value"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(a.small, a.gpus),
        "requested_steps": a.steps,
        "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": r["value"], "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(a) -> None:
    import ctypes

    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import _lib, meshgen

    world, rank, local = _dist()
    dev = torch.device("cuda", local)
    m, mu, lam, mask, fv = _mesh(a.small)
    mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
    b = ag.ModelBuilder(dtype=torch.float32)
    b.add_vertices(mesh)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    b.add_fixed(mesh)
    pot = ag.StableNeoHookean.from_pyvista(mesh)
    b.add_potential(pot)
    model = b.finalize()
    nt, nv = m.n_cells, m.n_points
    u0 = torch.tensor(np.where(mask, fv, 0.0), dtype=torch.float32, device=dev)

    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=2**30, rtol=0.0))
    fwd = ag.Forward(model, opt)
    solver = opt.solver(fwd.problem)
    solver.reset(u0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    for i in range(a.warmup):
        flush.fill_(i & 0xFF)
        solver.step()
    torch.cuda.synchronize(dev)
    if a.profile:
        # the three passes as plain launches (graph nodes that set a
        # conditional handle cannot be profiled individually), inside an
        # NVTX range for ncu's --nvtx-include "profile/"
        ms = (ctypes.c_float * 3)()
        torch.cuda.nvtx.range_push("profile")
        _lib.call("agb_solver_time_passes", solver.handle, a.steps, ctypes.c_void_p(flush.data_ptr()),
                  flush.numel(), ms, stream.cuda_stream)
        torch.cuda.synchronize(dev)
        torch.cuda.nvtx.range_pop()
        return
    clocks = ClockSampler(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    _barrier(world)
    torch.cuda.synchronize(dev)
    torch.cuda.nvtx.range_push("steps")  # the timed region, for ncu --nvtx-include "steps/"
    for i in range(a.steps):
        flush.fill_(i & 0xFF)
        ev[i][0].record(stream)
        solver.step()
        ev[i][1].record(stream)
    torch.cuda.synchronize(dev)
    torch.cuda.nvtx.range_pop()
    _barrier(world)
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in ev]
    value, total_s = _aggregate(world, a.steps, sum(step_ms) / 1e3)
    state = solver.read()
    if state.result != ag.Result.UNKNOWN_ERROR:
        raise RuntimeError(f"solver stopped inside the timed region: {state}")
    b_iter = nt * B_TET + nv * B_VERT

    # each pass alone, L2 flushed before each launch
    ms = (ctypes.c_float * 3)()
    _lib.call("agb_solver_time_passes", solver.handle, 20, ctypes.c_void_p(flush.data_ptr()), flush.numel(),
              ms, stream.cuda_stream)
    names = ("direction", "gradient", "vertex")
    per_launch = {  # algorithmic bytes of one launch of each pass
        "direction": nt * B_TET + nv * 4 * 12,
        "gradient": nt * B_TET + nv * 6 * 12,
        "vertex": nv * 12 * 11,
    }
    k = max(range(3), key=lambda i: ms[i])
    peak, peak_kind = _measured_peak()
    achieved = per_launch[names[k]] / (ms[k] * 1e-3) / 1e9
    traffic = None
    # dram bytes per launch from one ncu capture of this workload (the
    # small grid has none)
    tp = ROOT / "profiles" / "traffic_passes_snh_grid_50x50x120_1.5M.json"
    if tp.exists() and not a.small:
        rec = json.loads(tp.read_text())
        if rec.get("workload") == WORKLOAD:
            traffic = rec.get(names[k])

    # the headline solve: PNCG from the initial state to ||g||/||g0|| <= 1e-6
    solve_opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=20000, rtol=1e-6))
    solve_sv = solve_opt.solver(ag.ForwardProblem(model))
    solve_sv.reset(u0)
    solve_sv.iterate(1)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    solve_sv.reset(u0)
    solve_sv.iterate(20000)
    u32 = torch.empty_like(u0)
    ssol = solve_sv.read(u32)
    t_solve = time.perf_counter() - t0
    solve = {"rtol": 1e-6, "result": ssol.result.name, "iters": ssol.n_steps, "seconds": t_solve,
             "rel_grad": ssol.grad_norm / ssol.grad_norm_first, "iters_per_s": ssol.n_steps / t_solve}
    loop_us = loop_overhead_us(dev)
    accuracy = batched = adjoint = None
    if rank == 0 and not a.no_accuracy:
        try:
            accuracy = headline_accuracy(pot, model, m, mu, lam, mask, fv, u0, u32, dev)
        except Exception as e:  # noqa: BLE001
            accuracy = {"failed": f"{type(e).__name__}: {e}"}
    if rank == 0 and not a.no_forms:
        try:
            batched = batched_record(n=16 if a.small else 64)
        except Exception as e:  # noqa: BLE001
            batched = {"failed": f"{type(e).__name__}: {e}"}
        try:
            adjoint = adjoint_record(small=a.small)
        except Exception as e:  # noqa: BLE001
            adjoint = {"failed": f"{type(e).__name__}: {e}"}

    # end to end through the public host-buffer API
    e2e_opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=a.e2e_iters, rtol=0.0))
    e2e_solver = e2e_opt.solver(ag.ForwardProblem(model))
    u_host = torch.empty((nv, 3), dtype=torch.float32).pin_memory()
    base = u0.cpu()
    times = []
    for i in range(a.e2e_steps + 1):
        u_host.copy_(base)
        flush.fill_(i & 0xFF)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        sol = e2e_solver.minimize_host(u_host)
        t1 = time.perf_counter()
        if i > 0:
            times.append(t1 - t0)
        if sol.n_steps != a.e2e_iters:
            raise RuntimeError(f"e2e solve ran {sol.n_steps} iterations")
    e2e_value, e2e_s = _aggregate(world, a.e2e_iters, statistics.mean(times))
    e2e = {"value": e2e_value, "unit": "iter/s",
           "h2d_bytes_per_step": nv * 3 * 4, "d2h_bytes_per_step": nv * 3 * 4 + 160,
           "iters_per_step": a.e2e_iters, "ms_per_step": e2e_s * 1e3}

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        try:
            r = cpu_reference(10**6, a.cpu_budget, a.small)
            cpu = {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as e:  # noqa: BLE001
            cpu = {"value": None, "unit": "iter/s", "cores": None, "kind": "port", "sample": f"failed: {e}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * total_s / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": headline_config(a.small, world),
            "solver": {"step_form": "one CUDA graph per PNCG iteration",
                       "fp32_reference_correction": "on, FP64 refresh each 10x drop of ||g|| (solver default)"},
            "hbm_gbs_algorithmic": b_iter * value / world / 1e9,
            "roofline": {"bound": "hbm", "kernel": names[k], "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "bytes_per_launch": per_launch[names[k]], "ms_per_launch": ms[k]},
            "passes_ms": {n: ms[i] for i, n in enumerate(names)},
            "e2e": e2e,
            "solve_to_1e-6": solve,
            "loop_us_per_iter_320_tets": loop_us,
            "accuracy": accuracy,
            "batched": batched,
            "adjoint": adjoint,
            "cpu_baseline": cpu,
            "gpu_launches": solver.step_kernels() * a.steps,
            "clocks": clk,
            "step_ms_median": statistics.median(step_ms),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


ADJ_WORKLOAD = "snh_grid_24x24x48_138k_tets_stretch30_theta_mu"


def run_adjoint(a) -> None:
    """The adjoint workload: dL/dtheta for per-tet theta scaling mu, by the
    device adjoint (forward PNCG to 1e-7 in FP32, CG, material VJP), checked
    against central differences of the FP64 forward on `fd_cells` cells."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen
    from apple_gb300.adjoint import MaterialEquilibrium

    rng = np.random.default_rng(0)
    nx, ny, nz = (6, 6, 12) if a.small else (24, 24, 48)
    m = meshgen.grid(nx, ny, nz, h=1.0 / nx)
    lam0, mu0 = meshgen.lame_converter(E_MOD, NU)
    theta = rng.uniform(0.5, 2.0, m.n_cells)
    theta_star = rng.uniform(0.5, 2.0, m.n_cells)
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    top = meshgen.face_mask(m, 2, "max")
    mask[top] = True
    fv[top, 2] = STRETCH * m.points[:, 2].max()
    surf = np.zeros(m.n_points, bool)
    for ax in range(3):
        for side in ("min", "max"):
            surf |= meshgen.face_mask(m, ax, side)
    mesh = meshgen.TetMesh(m.points, m.cells)
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = fv
    lam = lam0 * np.ones(m.n_cells)
    crit32 = ag.ConvergenceCriteria(max_steps=200000, rtol=1e-7)
    crit64 = ag.ConvergenceCriteria(max_steps=200000, rtol=1e-10)
    p32 = MaterialEquilibrium(mesh, ag.StableNeoHookean, dtype=torch.float32, criteria=crit32, cg_rtol=1e-6)
    p64 = MaterialEquilibrium(mesh, ag.StableNeoHookean, dtype=torch.float64, criteria=crit64, cg_rtol=1e-10)
    dev = torch.device("cuda")
    si = torch.tensor(np.flatnonzero(surf), device=dev)

    target = p64.solve(mu0 * theta_star, lam)[si].clone()

    def loss(u):
        return 0.5 * float(((u.double()[si] - target) ** 2).sum())

    def gradient(prob, th):
        u = prob.solve(mu0 * th, lam)
        g = torch.zeros_like(u)
        g[si] = (u.double()[si] - target).to(u.dtype)
        d = prob.vjp(g)["mu"].double().cpu().numpy() * mu0  # dL/dtheta = dL/dmu * mu0
        return loss(u), d, dict(prob.timings), prob.stats

    gradient(p32, theta)  # warm-up (graph capture, kernel attributes)
    L32, d32, t32, s32 = gradient(p32, theta)
    L64, d64, t64, s64 = gradient(p64, theta)
    # central differences of FP64 forwards: one cell's dL/dtheta moves L by
    # ~1e-9 of itself at h = 1e-4 theta, so every perturbed solve starts from
    # the base u* and stops at the same absolute gradient norm (1e-12 of the
    # cold-start gradient), which keeps the solver's residual error equal on
    # both sides of each difference
    g_first = s64.forward.grad_norm_first
    crit_fd = ag.ConvergenceCriteria(max_steps=400000, rtol=0.0, atol=1e-12 * g_first)
    p_fd = MaterialEquilibrium(mesh, ag.StableNeoHookean, dtype=torch.float64, criteria=crit_fd)
    u_base = p_fd.solve(mu0 * theta, lam, u0=p64.solve(mu0 * theta, lam)).clone()
    base_stats = p_fd.stats.forward
    fd_solves = []

    def fd_loss(th):
        val = loss(p_fd.solve(mu0 * th, lam, u0=u_base))
        st = p_fd.stats.forward
        fd_solves.append((st.result.name, st.n_steps, st.grad_norm))
        return val

    # half the cells at random, half where |dL/dtheta| is largest (one cell's
    # effect on L is ~1e-8 of L for a random interior cell, near the noise of
    # the forward solves; the directional derivative below covers all cells)
    nfd = min(a.fd_cells, m.n_cells)
    rand_cells = rng.choice(m.n_cells, size=nfd - nfd // 2, replace=False)
    top_cells = [c for c in np.argsort(-np.abs(d64)) if c not in set(rand_cells)][: nfd // 2]
    cells = np.concatenate([rand_cells, np.asarray(top_cells, dtype=rand_cells.dtype)])
    # noise of L from the forward solves: the base point re-solved from a perturbed start
    u_pert = u_base + 1e-6 * torch.randn_like(u_base)
    noise = abs(loss(p_fd.solve(mu0 * theta, lam, u0=u_pert)) - loss(u_base))
    fd = []
    t_fd0 = time.perf_counter()
    for c in cells:
        h = 1e-3 * theta[c]
        vals = []
        for sgn in (1.0, -1.0):
            th = theta.copy()
            th[c] += sgn * h
            vals.append(fd_loss(th))
        fd.append((vals[0] - vals[1]) / (2 * h))
    t_fd = time.perf_counter() - t_fd0
    fd = np.asarray(fd)
    # directional derivative along a random direction v over all cells
    v = rng.normal(size=m.n_cells)
    hd = 1e-2
    lp = fd_loss(theta * (1.0 + hd * v))
    lm = fd_loss(theta * (1.0 - hd * v))
    fd_dir = (lp - lm) / (2 * hd)
    from collections import Counter
    fd_summary = {"base": [base_stats.result.name, base_stats.n_steps, base_stats.grad_norm / g_first],
                  "results": dict(Counter(r for r, _, _ in fd_solves)),
                  "max_rel_grad": max(gn for _, _, gn in fd_solves) / g_first,
                  "mean_steps": float(np.mean([n for _, n, _ in fd_solves])), "loss": L64,
                  "loss_noise": noise, "fd_signal_random_cells": float(np.median(np.abs(fd[: len(rand_cells)]))) * 2e-3}
    dir32 = float(np.dot(d32, v * theta))
    dir64 = float(np.dot(d64, v * theta))

    def rel(x, y):
        return float(np.linalg.norm(x - y) / np.linalg.norm(y))

    fwd32 = t32["forward"]
    adj32 = t32["adjoint"]
    line = {
        "metric": "adjoint dL/dtheta: s per full gradient (forward + adjoint) vs central differences",
        "config": {"workload": ADJ_WORKLOAD if not a.small else "snh_grid_6x6x12_adjoint", "n_tets": m.n_cells,
                   "n_vertices": m.n_points, "n_params": m.n_cells, "E": E_MOD, "nu": NU,
                   "loss": "0.5 ||u_surface - u_target||^2, u_target from hidden theta*",
                   "forward_rtol_f32": 1e-7, "cg_rtol_f32": 1e-6,
                   "fd_step": "1e-3 theta per cell, 1e-2 theta along a random direction (FP64 forwards from u*, "
                               "to 1e-12 of the cold-start gradient)"},
        "f32": {"forward_s": fwd32, "forward_iters": s32.forward.n_steps, "adjoint_s": adj32,
                "cg_iters": s32.cg.n_iter, "gradient_s": fwd32 + adj32,
                "rel_err_vs_fd": rel(d32[cells], fd), "rel_err_vs_fd_random": rel(d32[rand_cells], fd[: len(rand_cells)]),
                "rel_err_vs_fd_largest": rel(d32[cells[len(rand_cells):]], fd[len(rand_cells):]),
                "rel_err_vs_f64_adjoint": rel(d32, d64)},
        "f64": {"forward_s": t64["forward"], "forward_iters": s64.forward.n_steps, "adjoint_s": t64["adjoint"],
                "cg_iters": s64.cg.n_iter, "rel_err_vs_fd": rel(d64[cells], fd),
                "rel_err_vs_fd_random": rel(d64[rand_cells], fd[: len(rand_cells)]),
                "rel_err_vs_fd_largest": rel(d64[cells[len(rand_cells):]], fd[len(rand_cells):])},
        "fd": {"cells": int(len(cells)), "seconds": t_fd, "seconds_per_param": t_fd / max(len(cells), 1),
               "solves": fd_summary},
        "directional": {"fd": fd_dir, "f32": dir32, "f64": dir64, "rel_err_f32": abs(dir32 - fd_dir) / abs(fd_dir),
                        "rel_err_f64": abs(dir64 - fd_dir) / abs(fd_dir)},
        "adjoint_vs_plain": {
            "plain": "central differences of the plain forward, 2 solves per parameter",
            "plain_s_all_params_f32_est": 2 * m.n_cells * fwd32,
            "adjoint_s_f32": fwd32 + adj32,
            "speedup_est": 2 * m.n_cells * fwd32 / (fwd32 + adj32),
            "adjoint_over_forward": adj32 / fwd32,
        },
        "dtype": "f32 (and f64 check)", "data": "synthetic",
    }
    print(json.dumps(line), flush=True)


BATCH_WORKLOAD = "snh_batch_512_grids_4to40_cells_per_axis"
IRR_MAX_STEPS = 20000


def _batch_models(cases, dtype, tile_elems=0, workers=16):
    """Models of the batched workload, built on host threads (the C ABI set-up
    releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor

    import apple_gb300 as ag
    from apple_gb300 import meshgen

    def build(case):
        m, f = case
        pot = ag.StableNeoHookean.from_pyvista(m, dtype=dtype, tile_elems=tile_elems)
        b = ag.ModelBuilder(dtype=dtype)
        b.add_vertices(m)
        b.add_fixed(m)
        b.add_potential(pot)
        fm = meshgen.TetMesh(m.points, m.cells)
        fm.point_data["Force"] = f
        fm.point_data["GlobalPointId"] = np.arange(m.n_points)
        b.add_potential(ag.ExternalForce.from_pyvista(fm, dtype=dtype))
        model = b.finalize()
        model.warp_model.handle  # create the device model on this thread
        return model

    import numpy as np

    with ThreadPoolExecutor(workers) as ex:
        return list(ex.map(build, cases))


def run_batched(a) -> None:
    """The batched workload: all meshes in one batch (one graph launch per
    iteration of every running mesh) vs the plain per-mesh solve."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen
    from apple_gb300.batch import BatchedForward, autotune
    from oracle import fem_oracle as O

    n = 24 if a.small else a.n_meshes
    dims = (4, 12) if a.small else (4, 40)
    rng = np.random.default_rng(0)
    # 2.5 mm cells: objects of 1-10 cm, so gravity strains of E = 1e3..1e5 Pa stay moderate
    cases = [meshgen.batch_case(k, rng, dims=dims, h=1.0 / 400) for k in range(n)]
    crit = ag.ConvergenceCriteria(max_steps=50000, rtol=1e-6)
    dtype = torch.float32
    t0 = time.perf_counter()
    sub = [cases[i] for i in np.random.default_rng(1).choice(n, size=min(24, n), replace=False)]
    tune = autotune(lambda te: _batch_models(sub, dtype, te), iters=5, optimizer=ag.PNCG(crit))
    t_tune = time.perf_counter() - t0
    t0 = time.perf_counter()
    models = _batch_models(cases, dtype, tune.tile_elems)
    t_build = time.perf_counter() - t0
    bf = BatchedForward(models, ag.PNCG(crit), chunk_verts=tune.chunk_verts)
    n_points, n_cells = bf.info()
    bf.solve(max_steps=3)  # warm-up: graph capture
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bf.reset()
    bf.iterate(crit.max_steps)
    sols, us = bf.read()
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    # plain: every model on its own (reset + iterate graph + read), in sequence
    plain_u, plain_sols, t_plain = [], [], 0.0
    for mdl in models:
        opt = ag.PNCG(crit)
        fwd = ag.Forward(mdl, opt)
        opt.solver(fwd.problem)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        sol = fwd.step()
        torch.cuda.synchronize()
        t_plain += time.perf_counter() - t1
        plain_sols.append(sol)
        plain_u.append(fwd.state.u)
    diag = [float(np.linalg.norm(m.points.max(0) - m.points.min(0))) for m, _ in cases]
    err_bp = max(float((u.double() - v.double()).abs().max()) / d for u, v, d in zip(us, plain_u, diag))
    # FP64 oracle on the smallest meshes
    small = sorted(range(n), key=lambda k: cases[k][0].n_cells)[:4]
    err_o = []
    for k in small:
        m, f = cases[k]
        ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=m.cell_data["mu"],
                                       lam=m.cell_data["lambda"])
        om = O.Model(O.DofMap(m.n_points, m.point_data["FixedMask"], np.zeros((m.n_points, 3))), [ora],
                     O.ExternalForce(np.arange(m.n_points), f))
        u_ref, _ = O.solve_model(om, rtol=1e-10, max_steps=50000)
        err_o.append(float(np.abs(us[k].double().cpu().numpy() - u_ref).max()) / diag[k])
    iters = np.array([s.n_steps for s in sols])
    ok = sum(s.result == ag.Result.PRIMARY_SUCCESS for s in sols)
    ok_plain = sum(s.result == ag.Result.PRIMARY_SUCCESS for s in plain_sols)
    tet_iters = sum(m.n_cells * s.n_steps for (m, _), s in zip(cases, sols))
    conv = [k for k in range(n) if sols[k].result == ag.Result.PRIMARY_SUCCESS
            and plain_sols[k].result == ag.Result.PRIMARY_SUCCESS]
    err_bp_conv = max((float((us[k].double() - plain_u[k].double()).abs().max()) / diag[k] for k in conv),
                      default=None)
    stalled = [sols[k].grad_norm / sols[k].grad_norm_first for k in range(n)
               if sols[k].result != ag.Result.PRIMARY_SUCCESS]
    line = {
        "metric": "batched vs plain: seconds to solve every mesh to ||g||/||g0|| <= 1e-6",
        "config": {"workload": BATCH_WORKLOAD if not a.small else "snh_batch_24_grids_4to12", "n_meshes": n,
                   "n_tets": n_cells, "n_vertices": n_points, "dims_per_axis": list(dims),
                   "tile_elems": tune.tile_elems, "chunk_verts": tune.chunk_verts},
        "batched_s": t_batch, "plain_s": t_plain, "speedup": t_plain / t_batch,
        "batched_tet_iters_per_s": tet_iters / t_batch,
        "iters": {"mean": float(iters.mean()), "max": int(iters.max()), "min": int(iters.min())},
        "converged": {"batched": int(ok), "plain": int(ok_plain), "of": n},
        "max_diff_batched_vs_plain_over_diag": err_bp,
        "max_diff_batched_vs_plain_over_diag_converged": err_bp_conv,
        "not_converged_rel_grad_quantiles": (np.quantile(stalled, [0.0, 0.5, 1.0]).tolist() if stalled else None),
        "max_err_vs_fp64_oracle_over_diag": max(err_o) if err_o else None,
        "autotune": {"seconds": t_tune, "table_ms_per_iter": tune.table}, "build_s": t_build,
        "dtype": "f32", "data": "synthetic",
    }
    print(json.dumps(line), flush=True)


def _timed_steps(sv, steps, warmup, dev):
    import statistics

    import torch

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for i in range(warmup):
        flush.fill_(i & 0xFF)
        sv.step()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize(dev)
    for i in range(steps):
        flush.fill_(i & 0xFF)
        ev[i][0].record(stream)
        sv.step()
        ev[i][1].record(stream)
    torch.cuda.synchronize(dev)
    ms = [x.elapsed_time(y) for x, y in ev]
    return statistics.median(ms), sum(ms)


def _solve_case(model, u0, rtol, max_steps, dev):
    import apple_gb300 as ag
    import torch

    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=max_steps, rtol=rtol))
    sv = opt.solver(ag.ForwardProblem(model))
    sv.reset(u0)
    sv.iterate(1)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    sv.reset(u0)
    sv.iterate(max_steps)
    u = torch.empty_like(u0)
    sol = sv.read(u)
    return sol, time.perf_counter() - t0, u


def run_grid64(a) -> None:
    """The 64x64x96-cell grid (1,966,080 tets): iteration speed of ARAP (mu = 1) and
    stable Neo-Hookean in FP32 and FP64, and the FP32 energy / gradient / solution
    error against the FP64 oracle."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen
    from oracle import fem_oracle as O

    nx, ny, nz = (16, 16, 24) if a.small else (64, 64, 96)
    m = meshgen.grid(nx, ny, nz, h=1.0 / nx)
    lam, mu = meshgen.lame_converter(E_MOD, NU)
    mask = np.zeros((m.n_points, 3), bool)
    fv = np.zeros((m.n_points, 3))
    mask[meshgen.face_mask(m, 2, "min")] = True
    top = meshgen.face_mask(m, 2, "max")
    mask[top] = True
    fv[top, 2] = STRETCH * m.points[:, 2].max()
    dev = torch.device("cuda")
    out = {"metric": "PNCG iters/s on the 64x64x96 grid", "config": {
        "workload": "grid_64x64x96_1.97M_tets_stretch30" if not a.small else "grid_16x16x24", "n_tets": m.n_cells,
        "n_vertices": m.n_points, "E": E_MOD, "nu": NU, "arap_mu": 1.0}, "variants": {}}
    B_iter = {"snh": 64 * m.n_cells + 84 * m.n_points, "arap": 60 * m.n_cells + 84 * m.n_points}
    peak, _ = _measured_peak()
    for mat in ("snh", "arap"):
        for dtype in (torch.float32, torch.float64):
            mesh = meshgen.TetMesh(m.points, m.cells)
            if mat == "snh":
                mesh = ag.with_lame(mesh, mu, lam)
                cls = ag.StableNeoHookean
            else:
                mesh.cell_data["mu"] = np.ones(m.n_cells)
                cls = ag.Arap
            mesh.point_data["FixedMask"] = mask
            mesh.point_data["FixedValue"] = fv
            b = ag.ModelBuilder(dtype=dtype)
            b.add_vertices(mesh)
            b.add_fixed(mesh)
            b.add_potential(cls.from_pyvista(mesh, dtype=dtype))
            model = b.finalize()
            u0 = torch.tensor(np.where(mask, fv, 0.0), dtype=dtype, device=dev)
            opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=2**30, rtol=0.0))
            sv = opt.solver(ag.ForwardProblem(model))
            sv.reset(u0)
            steps = 30 if dtype == torch.float64 else 300
            med, tot = _timed_steps(sv, steps, 5, dev)
            key = f"{mat}_{'f32' if dtype == torch.float32 else 'f64'}"
            v = {"iters_per_s": steps / (tot / 1e3), "ms_per_iter_median": med,
                 "hbm_gbs_algorithmic": B_iter[mat] * steps / (tot / 1e3) / 1e9}
            v["frac_of_measured_hbm"] = v["hbm_gbs_algorithmic"] / peak
            if dtype == torch.float32:
                # FP32 vs FP64 oracle at the iterate reached after the timed steps
                u = torch.empty_like(u0)
                sv.read(u)
                u64 = u.double().cpu().numpy()
                ora = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN if mat == "snh" else O.Material.ARAP,
                                               m.points, m.cells, mu=mu if mat == "snh" else 1.0,
                                               lam=lam if mat == "snh" else None)
                pot = model.warp_model.potentials[next(iter(model.warp_model.potentials))]
                ev = pot.eval(u, fun=True, grad=True)
                e_ref = ora.fun(u64)
                g_ref = ora.grad(u64)
                v["energy_rel_err_vs_fp64_oracle"] = abs(ev["fun"].item() / e_ref - 1.0)
                v["grad_rel_l2_err_vs_fp64_oracle"] = float(np.linalg.norm(ev["grad"].double().cpu().numpy() - g_ref)
                                                            / np.linalg.norm(g_ref))
            out["variants"][key] = v
    print(json.dumps(out), flush=True)


def run_irregular(a) -> None:
    """The irregular workload: a seeded Delaunay ball (300k interior + 20k shell
    points, random vertex order, per-tet mu log-uniform in [1e3, 1e6], lambda =
    10 mu): PNCG iteration speed in FP32, and the bit-exact check that the
    Morton reorder and the tile colouring keep every cell's four corners."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen

    n_in, n_sh = (20000, 3000) if a.small else (300000, 20000)
    t0 = time.perf_counter()
    m = meshgen.ball(n_in, n_sh, seed=0)
    rng = np.random.default_rng(0)
    perm = rng.permutation(m.n_points)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(m.n_points)
    pts = m.points[perm]
    cells = inv[m.cells].astype(np.int32)
    t_mesh = time.perf_counter() - t0
    mu = np.exp(rng.uniform(np.log(1e3), np.log(1e6), cells.shape[0]))
    mesh = meshgen.TetMesh(pts, cells)
    mesh.cell_data["mu"] = mu
    mesh.cell_data["lambda"] = 10.0 * mu
    r = np.linalg.norm(pts, axis=1)
    mask = np.zeros((pts.shape[0], 3), bool)
    mask[pts[:, 2] < -0.9] = True  # a fixed cap
    mesh.point_data["FixedMask"] = mask
    mesh.point_data["FixedValue"] = np.zeros((pts.shape[0], 3))
    f = meshgen.lumped_gravity(mesh, 1000.0)
    b = ag.ModelBuilder()
    b.add_vertices(mesh)
    b.add_fixed(mesh)
    pot = ag.StableNeoHookean.from_pyvista(mesh)
    b.add_potential(pot)
    fm = meshgen.TetMesh(pts, cells)
    fm.point_data["Force"] = f
    fm.point_data["GlobalPointId"] = np.arange(pts.shape[0])
    b.add_potential(ag.ExternalForce.from_pyvista(fm))
    model = b.finalize()
    dev = torch.device("cuda")
    u0 = torch.zeros((pts.shape[0], 3), dtype=torch.float32, device=dev)
    opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=2**30, rtol=0.0))
    sv = opt.solver(ag.ForwardProblem(model))
    sv.reset(u0)
    med, tot = _timed_steps(sv, 300, 5, dev)
    # connectivity as stored after the Morton reorder and the colouring: every
    # cell keeps its corner set; the plan is the same when built again
    stored, h1 = pot.stored_cells()
    _, h2 = ag.StableNeoHookean.from_pyvista(mesh).stored_cells()
    exact = bool(np.array_equal(np.sort(stored, axis=1), np.sort(cells, axis=1)))
    sol, t_solve, _ = _solve_case(model, u0, 1e-6, IRR_MAX_STEPS, dev)
    nt, ntv = pot.info()
    line = {"metric": "PNCG iters/s on the irregular Delaunay ball",
            "config": {"workload": "snh_delaunay_ball_320k_points" if not a.small else "snh_delaunay_ball_small",
                       "n_tets": int(cells.shape[0]), "n_vertices": int(pts.shape[0]), "mu": "log-uniform [1e3, 1e6]",
                       "lambda": "10 mu", "load": "gravity (rho 1000, g 9.8), cap z < -0.9 fixed"},
            "iters_per_s": 300 / (tot / 1e3), "ms_per_iter_median": med,
            "hbm_gbs_algorithmic": (64 * cells.shape[0] + 84 * pts.shape[0]) * 300 / (tot / 1e3) / 1e9,
            "tiles": nt, "tile_vertices_per_vertex": ntv / pts.shape[0],
            "connectivity_exact": exact, "plan_hash": h1, "plan_rebuild_identical": h1 == h2, "mesh_s": t_mesh,
            "solve": {"rtol": 1e-6, "max_steps": IRR_MAX_STEPS, "result": sol.result.name, "iters": sol.n_steps,
                      "seconds": t_solve, "rel_grad": sol.grad_norm / sol.grad_norm_first}}
    print(json.dumps(line), flush=True)


def run_irregular_study(a) -> None:
    """Why the irregular workload converges slowly: the same Delaunay ball at a
    smaller size (20,000 + 3,000 points, the small irregular workload) solved
    by Jacobi-preconditioned PNCG in FP32 and FP64 on the GPU and by the FP64
    C restatement of the reference's PNCG on the host, with the workload's
    stiffness contrast (mu log-uniform over three decades) and with a uniform
    mu (the contrast's geometric mean); FP32 also with the reference-state
    correction refreshed at every 2x drop of ||g|| (default: 100x) and without
    it.  ||g|| / ||g0|| is recorded at fixed iteration counts."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen
    from oracle import build_c
    from oracle import fem_oracle as O

    m = meshgen.ball(20000, 3000, seed=0)
    rng = np.random.default_rng(0)
    pts, cells = m.points, np.asarray(m.cells, np.int32)
    mask = np.zeros((pts.shape[0], 3), bool)
    mask[pts[:, 2] < -0.9] = True
    f = meshgen.lumped_gravity(m, 1000.0)
    dev = torch.device("cuda")
    marks = (1000, 5000, 20000)
    c_marks = (1000, 5000)
    out = {"workload": "snh_delaunay_ball_small (20,000 + 3,000 points), gravity, cap z < -0.9 fixed",
           "n_tets": int(cells.shape[0]), "n_vertices": int(pts.shape[0]), "rel_grad_at": {}}
    mu_contrast = np.exp(rng.uniform(np.log(1e3), np.log(1e6), cells.shape[0]))
    for name, mu in (("mu_log_uniform_1e3_1e6", mu_contrast),
                     ("mu_uniform_geometric_mean", np.full(cells.shape[0], np.sqrt(1e3 * 1e6)))):
        rec = {}
        mesh = meshgen.TetMesh(pts, cells)
        mesh.cell_data["mu"] = mu
        mesh.cell_data["lambda"] = 10.0 * mu
        mesh.point_data["FixedMask"] = mask
        mesh.point_data["FixedValue"] = np.zeros((pts.shape[0], 3))
        for dt, refresh in ((torch.float32, -1.0), (torch.float32, 0.5), (torch.float32, 0.0), (torch.float64, -1.0)):
            b = ag.ModelBuilder(dtype=dt)
            b.add_vertices(mesh)
            b.add_fixed(mesh)
            b.add_potential(ag.StableNeoHookean.from_pyvista(mesh, dtype=dt))
            fm = meshgen.TetMesh(pts, cells)
            fm.point_data["Force"] = f
            fm.point_data["GlobalPointId"] = np.arange(pts.shape[0])
            b.add_potential(ag.ExternalForce.from_pyvista(fm, dtype=dt))
            sv = ag.PNCG(ag.ConvergenceCriteria(max_steps=10**6, rtol=0.0),
                         refresh_ratio=refresh).solver(ag.ForwardProblem(b.finalize()))
            sv.reset(torch.zeros((pts.shape[0], 3), dtype=dt, device=dev))
            done, traj = 0, {}
            for k in marks:
                sv.iterate(k - done)
                done = k
                st = sv.read()
                traj[k] = {"rel_grad": st.grad_norm / st.grad_norm_first, "result": st.result.name,
                           "iters": st.n_steps}
            key = "gpu_f64" if dt == torch.float64 else {-1.0: "gpu_f32", 0.5: "gpu_f32_refresh_0.5",
                                                          0.0: "gpu_f32_no_correction"}[refresh]
            rec[key] = traj
        dhdX, dV = O.region_compute_grad(pts, cells)
        cm = build_c.CModel(1, cells, dhdX, dV, mu, 10.0 * mu, pts.shape[0], mask=mask.astype(np.uint8), force=f)
        traj = {}
        for k in c_marks:
            _, st = cm.pncg(np.zeros((pts.shape[0], 3)), max_steps=k, rtol=0.0)
            traj[k] = {"rel_grad": st.grad_norm / st.grad_norm_first, "iters": int(st.n_steps)}
        rec["c_restatement_f64"] = traj
        out["rel_grad_at"][name] = rec
    print(json.dumps(out), flush=True)


def run_muscle(a) -> None:
    """The headline grid (stretch 30%) as a stable Neo-Hookean muscle with a
    random per-cell activation (|a| ~ 0.05) vs the same grid without it:
    PNCG iterations per second, and a solve to 1e-6."""
    import numpy as np
    import torch

    import apple_gb300 as ag
    from apple_gb300 import meshgen

    dev = torch.device("cuda")
    m, mu, lam, mask, fv = _mesh(a.small)
    act = 0.05 * np.random.default_rng(0).normal(size=(m.n_cells, 6))
    u0 = torch.tensor(np.where(mask, fv, 0.0), dtype=torch.float32, device=dev)
    out = {}
    for name, cls in (("stable_neo_hookean", ag.StableNeoHookean), ("muscle", ag.StableNeoHookeanMuscle)):
        mesh = ag.with_lame(meshgen.TetMesh(m.points, m.cells), mu, lam)
        if cls is ag.StableNeoHookeanMuscle:
            mesh.cell_data["activation"] = act
        mesh.point_data["FixedMask"] = mask
        mesh.point_data["FixedValue"] = fv
        b = ag.ModelBuilder()
        b.add_vertices(mesh)
        b.add_fixed(mesh)
        b.add_potential(cls.from_pyvista(mesh))
        model = b.finalize()
        opt = ag.PNCG(ag.ConvergenceCriteria(max_steps=2**30, rtol=0.0))
        sv = opt.solver(ag.ForwardProblem(model))
        sv.reset(u0)
        med, tot = _timed_steps(sv, 300, 5, dev)
        sol, t_solve, _ = _solve_case(model, u0, 1e-6, 20000, dev)
        out[name] = {"iters_per_s": 300 / (tot / 1e3), "ms_per_iter_median": med,
                     "solve": {"rtol": 1e-6, "result": sol.result.name, "iters": sol.n_steps, "seconds": t_solve}}
    out["muscle_over_plain_time_per_iter"] = out["stable_neo_hookean"]["iters_per_s"] / out["muscle"]["iters_per_s"]
    print(json.dumps({"metric": "PNCG iters/s, muscle vs plain stable Neo-Hookean",
                      "config": {"workload": WORKLOAD + ("_small" if a.small else ""), "n_tets": m.n_cells,
                                 "activation": "N(0, 0.05^2) per component, seed 0"}, **out}), flush=True)


def run_hbm_sizes(a) -> None:
    """Cold-L2 bandwidth of a plain read (torch sum) and copy (torch copy_) vs
    the bytes one launch moves: a launch of ~100 MB cannot reach the STREAM
    figure measured on GB-sized arrays (launch latency, ramp-up and drain
    are a fixed cost of each launch), which bounds what one solver pass of
    that size can reach."""
    import statistics

    import torch

    dev = torch.device("cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    rows = []
    for mb in (16, 45, 72, 100, 200, 500, 2000):
        n = mb * (1 << 20) // 4
        x = torch.ones(n, dtype=torch.float32, device=dev)
        y = torch.empty(n // 2, dtype=torch.float32, device=dev)
        out = {"mb": mb}
        for kind in ("read", "copy"):
            ts = []
            for r in range(9):
                flush.fill_(r)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                if kind == "read":
                    x.sum()
                else:
                    y.copy_(x[: n // 2])
                e1.record()
                torch.cuda.synchronize()
                if r >= 2:
                    ts.append(e0.elapsed_time(e1) * 1e3)
            us = statistics.median(ts)
            out[kind + "_us"] = round(us, 2)
            out[kind + "_gbs"] = round(mb * (1 << 20) / (us * 1e-6) / 1e9, 1)
        rows.append(out)
        del x, y
    peak, kind = _measured_peak()
    print(json.dumps({"metric": "cold-L2 bandwidth vs bytes per launch", "peak_gbs": peak, "peak_kind": kind,
                      "rows": rows, "note": "read = sum of a float32 array; copy = half the bytes read, half "
                                            "written; CUDA events around one launch, 256 MiB flush before each"}),
          flush=True)


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    elif a.config == "adjoint":
        run_adjoint(a)
    elif a.config == "batched":
        run_batched(a)
    elif a.config == "grid64":
        run_grid64(a)
    elif a.config == "hbm-sizes":
        run_hbm_sizes(a)
    elif a.config == "muscle":
        run_muscle(a)
    elif a.config == "irregular-study":
        run_irregular_study(a)
    elif a.config == "irregular":
        run_irregular(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
