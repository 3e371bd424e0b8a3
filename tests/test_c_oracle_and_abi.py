"""CPU checks: the C port of the reference path against the NumPy oracle, and
the C ABI library (loads, exports every declared symbol, host-only entry
points)."""

import ctypes
import pathlib
import re
import shutil
import subprocess

import numpy as np
import pytest

from apple_gb300 import _lib, meshgen
from oracle import build_c
from oracle import fem_oracle as O

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def c_lib():
    try:
        return build_c.load()
    except RuntimeError as e:  # no compiler
        pytest.skip(str(e))


def _pot(material, seed=0):
    rng = np.random.default_rng(seed)
    m = meshgen.grid(4, 3, 5)
    nt = m.n_cells
    mu = rng.uniform(0.5, 2.0, nt)
    lam = rng.uniform(1.0, 10.0, nt) if material == O.Material.STABLE_NEO_HOOKEAN else None
    pot = O.FemPotential.from_mesh(material, m.points, m.cells, mu=mu, lam=lam)
    X = m.points - m.points.mean(0)
    u = X @ (0.1 * rng.normal(size=(3, 3))).T + 0.002 * np.sin(X @ rng.normal(size=(3, 3)))
    p = rng.normal(size=u.shape)
    return m, pot, u, p


@pytest.mark.parametrize("material", [O.Material.ARAP, O.Material.STABLE_NEO_HOOKEAN])
def test_c_port_matches_numpy_oracle(material, c_lib):
    m, pot, u, p = _pot(material)
    cm = build_c.CModel(int(material), pot.cells, pot.dhdX, pot.dV, pot.mu, pot.lam, m.n_points)
    r = cm.eval(u, p)
    assert r["fun"] == pytest.approx(pot.fun(u), rel=1e-12)
    np.testing.assert_allclose(r["grad"], pot.grad(u), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["hess_diag"], pot.hess_diag(u), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(r["hess_prod"], pot.hess_prod(u, p), rtol=1e-10, atol=1e-12)
    assert r["hess_quad"] == pytest.approx(pot.hess_quad(u, p), rel=1e-10)


def test_c_port_pncg_matches_numpy_oracle(c_lib):
    m = meshgen.grid(3, 3, 4)
    lam, mu = meshgen.lame_converter(1e4, 0.45)
    pot = O.FemPotential.from_mesh(O.Material.STABLE_NEO_HOOKEAN, m.points, m.cells, mu=mu, lam=lam)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    f = meshgen.lumped_gravity(m, 1000.0)
    om = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [pot], O.ExternalForce(np.arange(m.n_points), f))
    u_ref, st_ref = O.solve_model(om, rtol=0.0, max_steps=25)
    cm = build_c.CModel(1, pot.cells, pot.dhdX, pot.dV, pot.mu, pot.lam, m.n_points, mask=mask, force=f)
    u, st = cm.pncg(np.zeros((m.n_points, 3)), max_steps=25, rtol=0.0)
    assert st.n_steps == 25
    np.testing.assert_allclose(u, u_ref, rtol=1e-9, atol=1e-12)


def test_embedded_vertex_known_answer_c_port(c_lib):
    import json

    d = json.loads((ROOT / "tests/golden/embedded_tetra.json").read_text())
    pts = np.asarray(d["points"])
    cells = np.asarray(d["cells"])
    dhdX, dV = O.region_compute_grad(pts, cells)
    mask = np.zeros((5, 3), np.uint8)
    mask[d["fixed_vertices"]] = 1
    u0 = np.zeros((5, 3))
    u0[d["fixed_value_vertex"]] = d["fixed_value"]
    cm = build_c.CModel(0, cells, dhdX, dV, np.ones(4), None, 5, mask=mask)
    u, st = cm.pncg(u0)
    assert st.result == 0
    np.testing.assert_allclose(u[d["expect_vertex"]], d["expect_u"], atol=d["atol"])


def _declared_symbols():
    h = (ROOT / "include/apple_gb300.h").read_text()
    return sorted(set(re.findall(r"^(?:int|void|const char\*)\s+(agb_\w+)\(", h, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    declared = _declared_symbols()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_lib.exported_symbols())


_STRUCTS = {"agb_pncg_params": _lib.PncgParams, "agb_pncg_stats": _lib.PncgStats,
            "agb_cg_params": _lib.CgParams, "agb_cg_stats": _lib.CgStats}


def test_ctypes_structs_match_the_header(tmp_path):
    """Every struct the Python layer passes through the C ABI has the
    header's size and field offsets (a C program built against the header
    prints them)."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "apple_gb300.h"', "int main(void) {"]
    for name, cls in _STRUCTS.items():
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(line.split()[:2]): int(line.split()[2]) for line in out if line}
    for name, cls in _STRUCTS.items():
        assert got[(name, "size")] == ctypes.sizeof(cls), name
        for field, _ in cls._fields_:
            assert got[(name, field)] == getattr(cls, field).offset, (name, field)
    # and the header declares no field the Python struct lacks
    h = (ROOT / "include/apple_gb300.h").read_text()
    for name, cls in _STRUCTS.items():
        body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", h, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        fields = re.findall(r"^\s*\w+\s+(\w+);", body, re.M)
        assert fields == [f for f, _ in cls._fields_], name


def test_region_compute_host_entry_point():
    m = meshgen.ball(800, 200, seed=3)
    from apple_gb300 import region

    dhdX, dV = region.region_compute(m.points, m.cells)
    d2, v2 = O.region_compute_grad(m.points, m.cells)
    np.testing.assert_allclose(dhdX, d2, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(dV, v2, rtol=1e-12)


def test_c_abi_rejects_bad_mesh_without_gpu():
    """Argument checks run before any device work."""
    import ctypes

    cells = np.array([[0, 1, 2, 7]], np.int32)
    pts = np.zeros((4, 3))
    dh = np.zeros((1, 4, 3))
    dv = np.zeros(1)
    with pytest.raises(_lib.AgbError, match="outside"):
        _lib.call("agb_region_compute", 1, cells.ctypes.data, 4, pts.ctypes.data, None, dh.ctypes.data,
                  dv.ctypes.data, ctypes.byref(ctypes.c_int32()))


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the built library every entry raises."""
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", tmp_path / "libapple_gb300.so")
    with pytest.raises(ImportError, match="no fallback"):
        _lib.load()
    with pytest.raises(ImportError):
        _lib.call("agb_version")
