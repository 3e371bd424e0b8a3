"""VTK XML unstructured-grid files (``.vtu``) without pyvista or VTK.

The reference reads its meshes and attributes with pyvista (``pv.read``) and
hands ``mesh.points``, the tetrahedra of ``mesh.cells_dict[VTK_TETRA]``,
``mesh.point_data`` (``FixedMask``, ``FixedValue``, ``GlobalPointId``,
``Force``) and ``mesh.cell_data`` (``mu``, ``lambda``, ``Fraction``,
``activation``) to the potentials (``warp/fem/_base.py:78-111``,
``common/attr_name.py:4-44``).  :func:`read` returns the same attributes in a
:class:`~apple_gb300.meshgen.TetMesh`, so a ``.vtu`` input goes straight into
``from_pyvista``; :func:`write` stores a mesh with its arrays (for instance the
solved displacement) for pyvista/ParaView.

Encodings follow the VTK XML file format: ``ascii``; ``binary`` (base64,
inline) and ``appended`` (``raw`` or ``base64``) data, each with a UInt32 or
UInt64 byte-count header, optionally zlib-compressed in blocks
(``vtkZLibDataCompressor``); little- or big-endian files (written
little-endian).  Only tetrahedra (cell type 10) are read as
cells; other cell types are skipped with their cell data.
"""

from __future__ import annotations

import base64
import xml.etree.ElementTree as ET
import zlib

import numpy as np

from .meshgen import TetMesh

VTK_TETRA = 10

_TYPES = {
    "Int8": np.int8, "UInt8": np.uint8, "Int16": np.int16, "UInt16": np.uint16,
    "Int32": np.int32, "UInt32": np.uint32, "Int64": np.int64, "UInt64": np.uint64,
    "Float32": np.float32, "Float64": np.float64,
}
_NAMES = {np.dtype(v).str[1:]: k for k, v in _TYPES.items()}


class _Ctx:
    def __init__(self, root: ET.Element, appended: bytes | None, appended_encoding: str):
        order = root.get("byte_order", "LittleEndian")
        if order not in ("LittleEndian", "BigEndian"):
            raise ValueError(f"unknown byte_order {order}")
        self.order = "<" if order == "LittleEndian" else ">"
        hdr = np.uint64 if root.get("header_type", "UInt32") == "UInt64" else np.uint32
        self.hdr = np.dtype(hdr).newbyteorder(self.order)
        self.hsize = np.dtype(self.hdr).itemsize
        comp = root.get("compressor")
        if comp not in (None, "", "vtkZLibDataCompressor"):
            raise ValueError(f"unsupported compressor {comp}")
        self.zlib = comp == "vtkZLibDataCompressor"
        self.appended = appended
        self.appended_encoding = appended_encoding
        self._text = None

    def _ints(self, b: bytes, n: int) -> list[int]:
        return [int(x) for x in np.frombuffer(b[: n * self.hsize], self.hdr)]

    def _block_header_len(self, first: bytes) -> int:
        return 3 + self._ints(first, 1)[0]  # nblocks, blocksize, lastsize, sizes...

    def decode_b64(self, text: str) -> bytes:
        """Inline ``binary`` data of one array."""
        return self._b64_at("".join(text.split()), 0)

    def _b64_at(self, text: str, pos: int) -> bytes:
        """One array's base64 data starting at ``pos``: the byte-count header
        and the data are encoded together, or as two streams (VTK encodes a
        compressed block header on its own); a separate header stream ends in
        padding, which a joint stream cannot have at that position."""
        b64len = lambda n: -(-n // 3) * 4  # noqa: E731
        hl = b64len(self.hsize)
        if not self.zlib:
            if text[pos + hl - 1] == "=":  # separate streams, or a joint one that ends here
                head = base64.b64decode(text[pos: pos + hl])
                n = self._ints(head, 1)[0]
                if len(head) >= self.hsize + n:
                    return head[self.hsize: self.hsize + n]
                return base64.b64decode(text[pos + hl: pos + hl + b64len(n)])[:n]
            n = self._ints(base64.b64decode(text[pos: pos + b64len(self.hsize + 1)]), 1)[0]
            raw = base64.b64decode(text[pos: pos + b64len(self.hsize + n)])
            return raw[self.hsize: self.hsize + n]
        nh = self._block_header_len(base64.b64decode(text[pos: pos + b64len(3 * self.hsize)]))
        hl = b64len(nh * self.hsize)
        head = base64.b64decode(text[pos: pos + hl])
        total = sum(self._ints(head[3 * self.hsize:], nh - 3))
        return self._inflate(head, base64.b64decode(text[pos + hl: pos + hl + b64len(total)]))

    def _inflate(self, head: bytes, body: bytes) -> bytes:
        nb, _, _ = self._ints(head, 3)
        sizes = self._ints(head[3 * self.hsize:], nb)
        out, pos = [], 0
        for s in sizes:
            out.append(zlib.decompress(body[pos: pos + s]))
            pos += s
        return b"".join(out)

    def decode_appended(self, offset: int) -> bytes:
        data = self.appended
        if self.appended_encoding == "raw":
            if not self.zlib:
                n = self._ints(data[offset:], 1)[0]
                return data[offset + self.hsize: offset + self.hsize + n]
            nh = self._block_header_len(data[offset:])
            head = data[offset: offset + nh * self.hsize]
            total = sum(self._ints(head[3 * self.hsize:], nh - 3))
            return self._inflate(head, data[offset + nh * self.hsize: offset + nh * self.hsize + total])
        if self._text is None:
            self._text = data.decode("ascii")
        return self._b64_at(self._text, offset)


def _array(ctx: _Ctx, el: ET.Element) -> np.ndarray:
    dt = np.dtype(_TYPES[el.get("type")]).newbyteorder(ctx.order)
    nc = int(el.get("NumberOfComponents", "1"))
    fmt = el.get("format", "ascii")
    if fmt == "ascii":
        a = np.array((el.text or "").split(), dtype=dt)
    elif fmt == "binary":
        a = np.frombuffer(ctx.decode_b64(el.text or ""), dtype=dt)
    elif fmt == "appended":
        a = np.frombuffer(ctx.decode_appended(int(el.get("offset"))), dtype=dt)
    else:
        raise ValueError(f"unknown DataArray format {fmt}")
    a = a.astype(a.dtype.newbyteorder("="))  # native order, a copy
    return a.reshape(-1, nc) if nc > 1 else a


def read(path) -> TetMesh:
    """Points, tetrahedra and their point / cell arrays of a ``.vtu`` file."""
    raw = open(path, "rb").read()
    appended, enc = None, "raw"
    i = raw.find(b"<AppendedData")
    if i >= 0:  # raw bytes may not be valid XML: cut them out before parsing
        j = raw.index(b">", i)
        tag = raw[i: j + 1].decode("ascii")
        enc = "base64" if 'encoding="base64"' in tag else "raw"
        u = raw.index(b"_", j) + 1
        k = raw.rfind(b"</AppendedData>")
        appended = raw[u:k]
        raw = raw[:i] + b"</VTKFile>"
    root = ET.fromstring(raw)
    if root.get("type") != "UnstructuredGrid":
        raise ValueError("not an UnstructuredGrid file")
    ctx = _Ctx(root, appended, enc)
    pieces = root.findall("./UnstructuredGrid/Piece")
    if len(pieces) != 1:
        raise ValueError("expected exactly one Piece")
    p = pieces[0]
    points = _array(ctx, p.find("./Points/DataArray")).astype(np.float64).reshape(-1, 3)
    cells_el = {el.get("Name"): el for el in p.findall("./Cells/DataArray")}
    conn = _array(ctx, cells_el["connectivity"]).astype(np.int64).ravel()
    offs = _array(ctx, cells_el["offsets"]).astype(np.int64).ravel()
    types = _array(ctx, cells_el["types"]).astype(np.int64).ravel()
    starts = np.concatenate([[0], offs[:-1]])
    tet = types == VTK_TETRA
    if np.any(offs[tet] - starts[tet] != 4):
        raise ValueError("tetra with a corner count other than 4")
    idx = starts[tet][:, None] + np.arange(4)
    cells = conn[idx].astype(np.int32) if idx.size else np.zeros((0, 4), np.int32)
    mesh = TetMesh(points, cells)
    for el in p.findall("./PointData/DataArray"):
        mesh.point_data[el.get("Name")] = _array(ctx, el)
    for el in p.findall("./CellData/DataArray"):
        mesh.cell_data[el.get("Name")] = _array(ctx, el)[tet]
    return mesh


def _encode(a: np.ndarray, fmt: str, compress: bool, hdr=np.uint64) -> tuple[str, bytes]:
    """(inline text, appended bytes) of one array."""
    data = np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
    if fmt == "ascii":
        if np.issubdtype(a.dtype, np.floating):
            return " ".join(repr(float(x)) for x in a.ravel()), b""
        return " ".join(str(int(x)) for x in a.ravel()), b""
    if compress:
        bs = 1 << 15
        blocks = [data[i: i + bs] for i in range(0, len(data), bs)] or [b""]
        comp = [zlib.compress(b) for b in blocks]
        head = np.array([len(blocks), bs, len(blocks[-1]), *map(len, comp)], hdr).tobytes()
        body = b"".join(comp)
        if fmt == "binary":
            return base64.b64encode(head).decode() + base64.b64encode(body).decode(), b""
        return "", head + body
    head = np.array([len(data)], hdr).tobytes()
    if fmt == "binary":
        return base64.b64encode(head + data).decode(), b""
    return "", head + data


def write(path, mesh, point_data: dict | None = None, cell_data: dict | None = None, *,
          fmt: str = "appended", compress: bool = True, encoding: str = "raw") -> None:
    """Write points, tetrahedra and arrays (``mesh.point_data`` / ``cell_data``
    merged with the extra dicts) as a ``.vtu``; ``fmt`` is ``ascii``, ``binary``
    or ``appended``, ``encoding`` (appended data) ``raw`` or ``base64``, and
    ``compress`` zlib-compresses binary data."""
    if fmt not in ("ascii", "binary", "appended") or encoding not in ("raw", "base64"):
        raise ValueError(f"unknown format {fmt} / encoding {encoding}")
    pts = np.asarray(mesh.points, np.float64).reshape(-1, 3)
    cells = np.asarray(mesh.cells, np.int64).reshape(-1, 4)
    pd = dict(getattr(mesh, "point_data", {}) or {})
    pd.update(point_data or {})
    cd = dict(getattr(mesh, "cell_data", {}) or {})
    cd.update(cell_data or {})
    compress = compress and fmt != "ascii"
    root = ET.Element("VTKFile", type="UnstructuredGrid", version="1.0", byte_order="LittleEndian",
                      header_type="UInt64")
    if compress:
        root.set("compressor", "vtkZLibDataCompressor")
    piece = ET.SubElement(ET.SubElement(root, "UnstructuredGrid"), "Piece",
                          NumberOfPoints=str(pts.shape[0]), NumberOfCells=str(cells.shape[0]))
    appended = []
    pos = 0

    def add(parent, name, a):
        nonlocal pos
        a = np.asarray(a)
        if a.dtype == np.bool_:
            a = a.astype(np.uint8)
        if a.dtype.str[1:] not in _NAMES:
            a = a.astype(np.float64)
        el = ET.SubElement(parent, "DataArray", type=_NAMES[a.dtype.str[1:]], format=fmt)
        if name:
            el.set("Name", name)
        if a.ndim > 1:
            el.set("NumberOfComponents", str(int(np.prod(a.shape[1:]))))
        text, blob = _encode(a, fmt, compress)
        if fmt == "appended" and encoding == "base64":  # the inline form's text, appended
            blob = _encode(a, "binary", compress)[0].encode("ascii")
        if fmt == "appended":
            el.set("offset", str(pos))
            appended.append(blob)
            pos += len(blob)
        else:
            el.text = text

    pde = ET.SubElement(piece, "PointData")
    for k, v in pd.items():
        add(pde, k, v)
    cde = ET.SubElement(piece, "CellData")
    for k, v in cd.items():
        add(cde, k, v)
    add(ET.SubElement(piece, "Points"), None, pts)
    ce = ET.SubElement(piece, "Cells")
    add(ce, "connectivity", cells.ravel())
    add(ce, "offsets", 4 * np.arange(1, cells.shape[0] + 1, dtype=np.int64))
    add(ce, "types", np.full(cells.shape[0], VTK_TETRA, np.uint8))
    xml = ET.tostring(root, encoding="unicode")
    with open(path, "wb") as f:
        if fmt != "appended":
            f.write(b'<?xml version="1.0"?>\n' + xml.encode())
            return
        head, tail = xml.rsplit("</VTKFile>", 1)
        f.write(b'<?xml version="1.0"?>\n' + head.encode() + f'<AppendedData encoding="{encoding}">_'.encode())
        f.write(b"".join(appended))
        f.write(b"</AppendedData></VTKFile>" + tail.encode())
