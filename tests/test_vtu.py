"""The .vtu reader / writer (no pyvista): every encoding round-trips the mesh
and its arrays bit for bit, UInt32 headers and one-byte arrays decode, only
tetrahedra are kept, and a file feeds the region precompute and the
potentials' from_pyvista."""

import base64
import zlib

import numpy as np
import pytest

from apple_gb300 import meshgen, vtu
from apple_gb300.region import Region


def _arrays(m, rng):
    pd = {"FixedMask": rng.random((m.n_points, 3)) < 0.3, "FixedValue": rng.normal(size=(m.n_points, 3)),
          "GlobalPointId": np.arange(m.n_points, dtype=np.int64)}
    cd = {"mu": rng.random(m.n_cells), "lambda": rng.random(m.n_cells).astype(np.float32),
          "activation": rng.normal(size=(m.n_cells, 6)), "Fraction": rng.random(m.n_cells)}
    return pd, cd


@pytest.mark.parametrize("fmt", ["ascii", "binary", "appended", "appended-base64"])
@pytest.mark.parametrize("compress", [False, True])
def test_round_trip(tmp_path, fmt, compress):
    rng = np.random.default_rng(0)
    m = meshgen.grid(20, 3, 2)  # > 32 KiB per array: several zlib blocks
    pd, cd = _arrays(m, rng)
    f = tmp_path / "m.vtu"
    enc = "base64" if fmt.endswith("base64") else "raw"
    vtu.write(f, m, pd, cd, fmt=fmt.split("-")[0], compress=compress, encoding=enc)
    r = vtu.read(f)
    np.testing.assert_array_equal(r.points, m.points)
    np.testing.assert_array_equal(r.cells, m.cells)
    for k, v in pd.items():
        np.testing.assert_array_equal(r.point_data[k], np.asarray(v).astype(r.point_data[k].dtype))
    for k, v in cd.items():
        np.testing.assert_array_equal(r.cell_data[k].reshape(np.shape(v)), v)


def _uint32_file(arrays, joint: bool, big_endian: bool = False, compress: bool = False) -> str:
    """A hand-assembled inline-binary file with UInt32 headers (in the
    file's byte order, as is its data; compressed: one zlib block per array,
    its header encoded on its own as VTK writes it)."""
    o = ">" if big_endian else "<"

    def enc(a):
        data = a.astype(a.dtype.newbyteorder(o)).tobytes()
        if compress:
            z = zlib.compress(data)
            head = np.array([1, len(data), len(data), len(z)], o + "u4").tobytes()
            return base64.b64encode(head).decode() + base64.b64encode(z).decode()
        head = np.array([len(data)], o + "u4").tobytes()
        if joint:
            return base64.b64encode(head + data).decode()
        return base64.b64encode(head).decode() + base64.b64encode(data).decode()

    pts, conn, offs, types, mu = arrays
    order = "BigEndian" if big_endian else "LittleEndian"
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    return f"""<?xml version="1.0"?>
<VTKFile type="UnstructuredGrid" version="0.1" byte_order="{order}" header_type="UInt32"{comp}>
 <UnstructuredGrid><Piece NumberOfPoints="{len(pts)}" NumberOfCells="{len(types)}">
  <CellData><DataArray type="Float64" Name="mu" format="binary">{enc(mu)}</DataArray></CellData>
  <Points><DataArray type="Float32" NumberOfComponents="3" format="binary">{enc(pts)}</DataArray></Points>
  <Cells>
   <DataArray type="Int32" Name="connectivity" format="binary">{enc(conn)}</DataArray>
   <DataArray type="Int32" Name="offsets" format="binary">{enc(offs)}</DataArray>
   <DataArray type="UInt8" Name="types" format="binary">{enc(types)}</DataArray>
  </Cells>
 </Piece></UnstructuredGrid>
</VTKFile>
"""


@pytest.mark.parametrize("joint", [True, False])
def test_uint32_headers_and_one_byte_arrays(tmp_path, joint):
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    arrays = (pts, np.array([0, 1, 2, 3], np.int32), np.array([4], np.int32), np.array([10], np.uint8),
              np.array([2.5]))
    f = tmp_path / "one.vtu"
    f.write_text(_uint32_file(arrays, joint))
    r = vtu.read(f)
    np.testing.assert_array_equal(r.cells, [[0, 1, 2, 3]])
    np.testing.assert_array_equal(r.points, pts.astype(np.float64))
    np.testing.assert_array_equal(r.cell_data["mu"], [2.5])


@pytest.mark.parametrize("joint,compress", [(True, False), (False, False), (False, True)])
def test_big_endian_files(tmp_path, joint, compress):
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float32) * 0.75
    conn = np.array([0, 1, 2, 3, 1, 2, 3, 4], np.int32)
    arrays = (pts, conn, np.array([4, 8], np.int32), np.array([10, 10], np.uint8), np.array([2.5, -1.25]))
    f = tmp_path / "be.vtu"
    f.write_text(_uint32_file(arrays, joint, big_endian=True, compress=compress))
    r = vtu.read(f)
    np.testing.assert_array_equal(r.cells, [[0, 1, 2, 3], [1, 2, 3, 4]])
    np.testing.assert_array_equal(r.points, pts.astype(np.float64))
    np.testing.assert_array_equal(r.cell_data["mu"], [2.5, -1.25])
    assert r.cell_data["mu"].dtype.isnative and r.points.dtype.isnative


def test_only_tetrahedra_are_kept(tmp_path):
    """A triangle (type 5) among the cells is skipped with its cell data."""
    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float32)
    conn = np.array([0, 1, 2, 3, 1, 2, 4, 1, 2, 3, 4], np.int32)
    offs = np.array([4, 7, 11], np.int32)
    types = np.array([10, 5, 10], np.uint8)
    mu = np.array([1.0, 9.0, 3.0])
    f = tmp_path / "mixed.vtu"
    f.write_text(_uint32_file((pts, conn, offs, types, mu), True))
    r = vtu.read(f)
    np.testing.assert_array_equal(r.cells, [[0, 1, 2, 3], [1, 2, 3, 4]])
    np.testing.assert_array_equal(r.cell_data["mu"], [1.0, 3.0])


def test_file_feeds_the_region_precompute(tmp_path):
    m = meshgen.grid(3, 3, 3)
    f = tmp_path / "g.vtu"
    vtu.write(f, m, cell_data={"mu": np.full(m.n_cells, 2.0), "lambda": np.full(m.n_cells, 5.0)})
    region = Region.from_pyvista(vtu.read(f), grad=True)
    assert region.dV.sum() == pytest.approx(m.volume(), rel=1e-12)
