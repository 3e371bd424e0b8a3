"""Generate ``reference_elements.npz``: golden vectors of the reference's own
element kernels, run unmodified on NumPy.

The reference (liblaf/apple) writes its kernels in Warp's Python DSL.  Warp,
JAX and the reference's helper packages are not installed here, but the
kernel and function bodies are plain Python.  This script loads the
reference's own source files, unchanged, with ``warp_numpy.py`` standing in
for ``warp`` and small stubs for the packages they import only for types or
class decoration (``liblaf.jarp``, ``jaxtyping``, ``pyvista``, ``felupe``;
``jax.numpy`` is NumPy itself).  What runs is the reference's code:

* ``jax/fem/region/_region.py:84-108`` ``Region.compute_grad`` with the
  reference's ``ElementTetra`` (``jax/fem/element/_tetra.py``) and 1-point
  ``QuadratureTetra`` (``jax/fem/quadrature/_tetra.py``): dhdX and dV;
* ``warp/fem/_base.py`` kernels built by ``make_*_kernel`` for each material
  (the per-(tet, qp) bodies with dV weighting, the clamps and the scatter):
  ``_deformation_gradient_kernel``, energy density, first Piola-Kirchhoff,
  fun, grad, hess_diag, hess_prod, hess_quad;
* the materials ``warp/fem/_stable_neo_hookean.py``,
  ``_stable_neo_hookean_muscle.py`` and ``_arap.py``, and everything they
  call in ``warp/fem/func/*.py`` and ``warp/math/*.py``.

ARAP's hess_prod kernel is recorded as the reference computes it (its
``_arap.py:55-56`` passes ``(dhdX, p)`` to ``h4_prod`` / ``h5_prod``, whose
signatures are ``(p, dhdX, ...)``), and, as ``arap_hess_prod_intended``, by
the same kernel template over a hess_prod that calls the reference's own
``h4_prod`` / ``h5_prod`` in their declared argument order.

``wp.svd3`` is compiled Warp code outside the reference tree; the stand-in's
LAPACK SVD is rotation-variant, and every golden F is non-inverted with
distinct singular values, where ARAP's results do not depend on the SVD's
sign convention.

Usage (only where the reference tree is present; tests read the .npz):

    python tests/golden/make_elem_golden.py <path-to-liblaf-apple>

or with ``APPLE_REFERENCE_ROOT`` set.
"""

from __future__ import annotations

import importlib
import os
import pathlib
import sys
import types
from typing import Any

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
OUT = HERE / "reference_elements.npz"
SEED = 20260516


class _Sub:
    """A name used only in annotations: subscriptable, callable, a base class."""

    def __class_getitem__(cls, item):
        return cls

    def __init__(self, *a, **k):
        pass


def _identity_decorator(*args, **kw):
    if len(args) == 1 and callable(args[0]) and not kw:
        return args[0]
    return lambda obj: obj


def _field(*args, default=None, **kw):
    return default


def _module(name: str, path: pathlib.Path | None = None, **attrs) -> types.ModuleType:
    m = types.ModuleType(name)
    if path is not None:
        m.__path__ = [str(path)]
    m.__dict__.update(attrs)
    sys.modules[name] = m
    parent, _, leaf = name.rpartition(".")
    if parent in sys.modules:
        setattr(sys.modules[parent], leaf, m)
    return m


def _export(pkg: types.ModuleType, submodules: list[str]) -> None:
    """Import the package's real submodules and lift their public names, as the
    reference's lazy ``__init__.pyi`` stubs do."""
    for sub in submodules:
        mod = importlib.import_module(f"{pkg.__name__}.{sub}")
        for k, v in vars(mod).items():
            if not k.startswith("_") and not isinstance(v, types.ModuleType):
                setattr(pkg, k, v)


def install(ref_root: pathlib.Path) -> types.SimpleNamespace:
    """Load the reference's element code over the stand-ins; returns its modules."""
    src = ref_root / "src" / "liblaf"
    apple = src / "apple"
    if not (apple / "warp" / "fem" / "_base.py").is_file():
        raise SystemExit(f"{ref_root} does not look like a liblaf/apple checkout")
    sys.path.insert(0, str(HERE))
    import warp_numpy

    sys.modules["warp"] = warp_numpy
    # third-party packages imported for types, decoration or unused code paths
    _module("jax", numpy=np, ensure_compile_time_eval=None, jacobian=None, hessian=None)
    sys.modules["jax.numpy"] = np
    _module("jaxtyping", Array=_Sub, Float=_Sub, Integer=_Sub)
    _module("pyvista", DataObject=_Sub, DataSet=_Sub, DataSetAttributes=_Sub)
    _module("felupe")
    _module("felupe.quadrature", Scheme=_Sub, Tetrahedron=_Sub)
    # liblaf.jarp: attrs / JAX-pytree decoration and Warp type aliases only
    _module("liblaf", src)
    _module("liblaf.jarp", define=_identity_decorator, frozen_static=_identity_decorator,
            struct=_identity_decorator, field=_field, array=_field, static=_field)
    _module("liblaf.jarp.warp")
    _module("liblaf.jarp.warp.types", floating=Any, mat43=Any, mat33=Any, vector=lambda *a, **k: Any)
    # liblaf.apple: real source files; the package __init__ files (lazy loaders
    # that would import everything) are replaced by these namespace modules
    _module("liblaf.apple", apple)
    _module("liblaf.apple.common", ACTIVATION=types.SimpleNamespace(value="activation", vtk="activation"),
            LAMBDA=types.SimpleNamespace(value="lambda_", vtk="lambda"),
            MU=types.SimpleNamespace(value="mu", vtk="mu"))
    _module("liblaf.apple.jax", apple / "jax")
    fem_j = _module("liblaf.apple.jax.fem", apple / "jax" / "fem")
    _export(_module("liblaf.apple.jax.fem.quadrature", apple / "jax" / "fem" / "quadrature"), ["_scheme", "_tetra"])
    _export(_module("liblaf.apple.jax.fem.element", apple / "jax" / "fem" / "element"), ["_element", "_tetra"])
    _module("liblaf.apple.jax.fem.geometry", Geometry=_Sub)
    _export(_module("liblaf.apple.jax.fem.region", apple / "jax" / "fem" / "region"), ["_region"])
    fem_j.Region = sys.modules["liblaf.apple.jax.fem.region"].Region
    _module("liblaf.apple.warp", apple / "warp")
    _module("liblaf.apple.warp.model", WarpPotential=type("WarpPotential", (), {}))
    _export(_module("liblaf.apple.warp.math", apple / "warp" / "math"), ["_misc", "_rotation"])
    _module("liblaf.apple.warp.fem", apple / "warp" / "fem")
    _export(_module("liblaf.apple.warp.fem.func", apple / "warp" / "fem" / "func"),
            ["_deformation", "_gradient", "_identity", "_misc", "_hess_diag", "_hess_prod", "_hess_quad"])
    _module("liblaf.apple.warp.fem.utils")
    ns = types.SimpleNamespace(
        wp=warp_numpy,
        region=sys.modules["liblaf.apple.jax.fem.region"],
        element=sys.modules["liblaf.apple.jax.fem.element"],
        quadrature=sys.modules["liblaf.apple.jax.fem.quadrature"],
        func=sys.modules["liblaf.apple.warp.fem.func"],
        math=sys.modules["liblaf.apple.warp.math"],
        base=importlib.import_module("liblaf.apple.warp.fem._base"),
        snh=importlib.import_module("liblaf.apple.warp.fem._stable_neo_hookean"),
        muscle=importlib.import_module("liblaf.apple.warp.fem._stable_neo_hookean_muscle"),
        arap=importlib.import_module("liblaf.apple.warp.fem._arap"),
    )
    return ns


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------
def _independent_tets(rng, n: int):
    """n tets with their own four vertices each: random rotation, scale and
    shear of the unit right tet, so every cell's dhdX differs."""
    base = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    pts = []
    for _ in range(n):
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        A = Q @ np.diag(rng.uniform(0.5, 2.0, 3)) @ (np.eye(3) + 0.2 * rng.normal(size=(3, 3)))
        if np.linalg.det(A) < 0:
            A[:, 0] = -A[:, 0]
        pts.append(base @ A.T + rng.normal(size=3))
    points = np.concatenate(pts)
    cells = np.arange(4 * n, dtype=np.int32).reshape(n, 4)
    return points, cells


def _grid():
    sys.path.insert(0, str(ROOT))
    from apple_gb300 import meshgen

    m = meshgen.grid(2, 2, 2)
    return np.asarray(m.points, np.float64), np.asarray(m.cells, np.int32)


def _deformation(rng, points):
    X = points - points.mean(0)
    return X @ (0.15 * rng.normal(size=(3, 3))).T + 0.02 * np.sin(3.0 * X @ rng.normal(size=(3, 3)))


# ---------------------------------------------------------------------------
# runs of the reference's kernels
# ---------------------------------------------------------------------------
def _region(ref, points, cells):
    """dhdX, dV by the reference's Region.compute_grad (jnp = NumPy)."""
    obj = types.SimpleNamespace(element=ref.element.ElementTetra(), quadrature=ref.quadrature.QuadratureTetra(),
                                points=points, cells_local=cells)
    ref.region.Region.compute_grad(obj)
    return np.asarray(obj.dhdX, np.float64), np.asarray(obj.dV, np.float64)


def _run(ref, cls, kernel, n_out, inputs, out_shape, inner):
    wp = ref.wp
    out = wp.Array(np.zeros(out_shape), inner_ndim=inner)
    wp.launch(kernel, dim=n_out, inputs=inputs, outputs=[out])
    return out.data


def _arap_hess_prod_intended(ref):
    """The reference's hess_prod kernel template over ARAP's intended H p:
    _arap.py:43-58 with h4_prod / h5_prod called in their declared order
    (p, dhdX, ...) (func/_hess_prod.py:38-55)."""
    wp, func, math = ref.wp, ref.func, ref.math

    @wp.func
    def hess_prod(F, p, dhdX, materials, cid):
        mu = materials.mu[cid]
        U, sigma, V = math.svd_rv(F)
        h4 = func.h4_prod(p, dhdX, U, sigma, V, clamp_lambda=True)
        h5 = func.h5_prod(p, dhdX)
        return F.dtype(0.5) * mu * (-F.dtype(2.0) * h4 + h5)

    return ref.base.WarpPotentialFem.make_hess_prod_kernel(hess_prod)


def evaluate(ref, cls, points, cells, u, p, mu, lam, act):
    wp = ref.wp
    nc, nv = cells.shape[0], points.shape[0]
    dhdX, dV = _region(ref, points, cells)
    region = types.SimpleNamespace(cells=wp.Array(cells, inner_ndim=1, dtype=np.int32),
                                   dhdX=wp.Array(dhdX, inner_ndim=2), dV=wp.Array(dV))
    materials = types.SimpleNamespace(mu=wp.Array(mu), lambda_=wp.Array(lam), activation=wp.Array(act, inner_ndim=1))
    U = wp.Array(u, inner_ndim=1)
    P = wp.Array(p, inner_ndim=1)
    dim = (nc, 1)
    r = {"dhdX": dhdX[:, 0], "dV": dV[:, 0]}
    r["F"] = _run(ref, cls, ref.base.WarpPotentialFem.deformation_gradient_kernel, dim,
                  [U, region.cells, region.dhdX], (nc, 1, 3, 3), 2)[:, 0]
    r["psi"] = _run(ref, cls, cls.energy_density_kernel, dim, [U, region.cells, region.dhdX, materials],
                    (nc, 1), 0)[:, 0]
    r["pk1"] = _run(ref, cls, cls.first_piola_kirchhoff_kernel, dim, [U, region.cells, region.dhdX, materials],
                    (nc, 1, 3, 3), 2)[:, 0]
    r["fun"] = _run(ref, cls, cls.fun_kernel, dim, [U, region, materials], (1,), 0)
    r["grad"] = _run(ref, cls, cls.grad_kernel, dim, [U, region, materials], (nv, 3), 1)
    r["hess_diag"] = _run(ref, cls, cls.hess_diag_kernel, dim, [U, region, materials], (nv, 3), 1)
    r["hess_prod"] = _run(ref, cls, cls.hess_prod_kernel, dim, [U, P, region, materials], (nv, 3), 1)
    r["hess_quad"] = _run(ref, cls, cls.hess_quad_kernel, dim, [U, P, region, materials], (1,), 0)
    if cls is ref.arap.Arap:
        r["arap_hess_prod_intended"] = _run(ref, cls, _arap_hess_prod_intended(ref), dim, [U, P, region, materials],
                                            (nv, 3), 1)
    return r


def main(ref_root: str) -> None:
    ref = install(pathlib.Path(ref_root))
    rng = np.random.default_rng(SEED)
    meshes = {"tets": _independent_tets(rng, 24), "grid": _grid()}
    classes = {"snh": ref.snh.StableNeoHookean, "muscle": ref.muscle.StableNeoHookeanMuscle, "arap": ref.arap.Arap}
    out: dict[str, np.ndarray] = {}
    for mname, (points, cells) in meshes.items():
        nc, nv = cells.shape[0], points.shape[0]
        out[f"{mname}__points"] = points
        out[f"{mname}__cells"] = cells
        for cname, cls in classes.items():
            for attempt in range(100):  # non-inverted F with distinct singular values
                u = _deformation(rng, points)
                F = np.eye(3) + np.einsum("cai,caj->cij", u[cells], _region(ref, points, cells)[0][:, 0])
                s = np.linalg.svd(F, compute_uv=False)
                if np.linalg.det(F).min() > 0.2 and np.diff(s, axis=1).__abs__().min() > 1e-3:
                    break
            else:
                raise RuntimeError("no admissible deformation")
            p = rng.normal(size=(nv, 3))
            mu = rng.uniform(0.5, 2.0, nc) * (1.0e3 if cname != "arap" else 1.0)
            lam = rng.uniform(2.0, 20.0, nc) * (1.0e3 if cname != "arap" else 0.0)
            act = 0.1 * rng.normal(size=(nc, 6)) if cname == "muscle" else np.zeros((nc, 6))
            r = evaluate(ref, cls, points, cells, u, p, mu, lam, act)
            key = f"{mname}__{cname}__"
            out[key + "u"] = u
            out[key + "p"] = p
            out[key + "mu"] = mu
            out[key + "lambda"] = lam
            out[key + "activation"] = act
            for k, v in r.items():
                out[key + k] = np.asarray(v, np.float64)
    out["meta__source"] = np.array(
        "liblaf/apple warp/fem/_base.py kernels (make_*_kernel), _stable_neo_hookean.py, "
        "_stable_neo_hookean_muscle.py, _arap.py, warp/fem/func/*.py, warp/math/*.py, "
        "jax/fem/region/_region.py:84-108 -- run unmodified over tests/golden/warp_numpy.py")
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("APPLE_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_elem_golden.py <path-to-liblaf-apple> (or set APPLE_REFERENCE_ROOT)")
    main(root)
