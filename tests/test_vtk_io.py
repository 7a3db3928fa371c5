"""VTK XML output and input without VTK (no GPU needed).

The writer follows rti's vtp_writer (io/vtp_writer.hpp: ASCII PolyData; cell
arrays Normals, radius, value, exposed-area, hitcnt, relative-error,
variance-of-variance; metadata as string field arrays); the readers follow
io/vtp_point_cloud_reader.hpp and io/vtp_triangle_reader.hpp.  Input files in
the other encodings VTK writes (inline base64, appended raw and base64, zlib
blocks) are generated here from the VTK XML format description.
"""
import base64
import os
import struct
import xml.etree.ElementTree as ET
import zlib

import numpy as np
import pytest

from rti_gb300 import RtgError, vtk

RNG = np.random.default_rng(3)


def _discs(n=7):
    p = RNG.normal(size=(n, 3)).astype(np.float32)
    nrm = RNG.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    r = RNG.uniform(0.01, 0.1, n).astype(np.float32)
    return p, nrm.astype(np.float32), r


def _cell_arrays(path):
    root = ET.parse(path).getroot()
    piece = root.find("PolyData/Piece")
    out = {}
    for da in piece.find("CellData"):
        vals = np.array(da.text.split(), dtype=np.float64)
        out[da.get("Name")] = (da.get("type"), int(da.get("NumberOfComponents", "1")), vals)
    return root, piece, out


def _field(root):
    out = {}
    for a in root.find("PolyData/FieldData"):
        codes = [int(x) for x in a.text.split()]
        assert codes[-1] == 0
        out[a.get("Name")] = bytes(codes[:-1]).decode()
    return out


def test_disc_writer_layout_and_values(tmp_path):
    p, n, r = _discs()
    s1 = RNG.random(7)
    cnt = RNG.integers(0, 2 ** 40, 7).astype(np.uint64)
    area = RNG.random(7).astype(np.float32)
    rel, vov = RNG.random(7), RNG.random(7)
    f = tmp_path / "d.vtp"
    meta = {"running-time[ns]": "123", "cmd": "rtg --infile a.vtp & <x>", "geo-name": "discs"}
    vtk.write_vtp_discs(str(f), p, n, r, value=s1, hitcnt=cnt, exposed_area=area, relative_error=rel, vov=vov,
                        metadata=meta)
    root, piece, ca = _cell_arrays(f)
    assert root.get("type") == "PolyData"
    assert piece.get("NumberOfPoints") == "7" and piece.get("NumberOfVerts") == "7"
    assert piece.get("NumberOfPolys") == "0"
    assert piece.find("CellData").get("Normals") == "Normals"
    assert list(ca) == ["Normals", "radius", "value", "exposed-area", "hitcnt", "relative-error",
                        "variance-of-variance"]
    assert ca["Normals"][1] == 3
    np.testing.assert_array_equal(ca["Normals"][2].astype(np.float32), n.ravel())
    np.testing.assert_array_equal(ca["radius"][2].astype(np.float32), r)
    np.testing.assert_array_equal(ca["value"][2], s1)
    np.testing.assert_array_equal(ca["exposed-area"][2].astype(np.float32), area)
    assert ca["hitcnt"][0] == "UInt64"
    assert [int(x) for x in ET.parse(f).getroot().find("PolyData/Piece/CellData")[4].text.split()] == \
        [int(c) for c in cnt]
    np.testing.assert_array_equal(ca["relative-error"][2], rel)
    np.testing.assert_array_equal(ca["variance-of-variance"][2], vov)
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=np.float32)
    np.testing.assert_array_equal(pts, p.ravel())
    verts = piece.find("Verts")
    assert [int(x) for x in verts[0].text.split()] == list(range(7))
    assert [int(x) for x in verts[1].text.split()] == list(range(1, 8))
    assert _field(root) == meta


def test_disc_round_trip_through_the_reader(tmp_path):
    p, n, r = _discs(50)
    f = tmp_path / "rt.vtp"
    vtk.write_vtp_discs(str(f), p, n, r, value=np.zeros(50))
    p2, n2, r2 = vtk.read_point_cloud(str(f))
    np.testing.assert_array_equal(p2, p)
    np.testing.assert_allclose(n2, n, rtol=0, atol=2e-7)
    np.testing.assert_array_equal(r2, r)


def test_triangle_writer_and_reader(tmp_path):
    v = RNG.random((9, 3)).astype(np.float32)
    t = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8], [0, 4, 8]], np.uint32)
    f = tmp_path / "t.vtp"
    vtk.write_vtp_triangles(str(f), v, t, value=np.arange(4.0), hitcnt=np.arange(4))
    root, piece, ca = _cell_arrays(f)
    assert piece.get("NumberOfPolys") == "4" and piece.get("NumberOfVerts") == "0"
    assert list(ca) == ["value", "hitcnt"]
    conn = [int(x) for x in piece.find("Polys")[0].text.split()]
    assert conn == t.ravel().tolist()
    v2, t2 = vtk.read_triangles(str(f))
    np.testing.assert_array_equal(v2, v)
    np.testing.assert_array_equal(t2, t)


# ---- input in the other encodings -------------------------------------------

def _enc_block(raw: bytes, header: str, compress: bool, b64: bool, joint: bool = True):
    """One DataArray payload: VTK's [header][data] (or zlib blocks)."""
    hf = "<I" if header == "UInt32" else "<Q"
    if not compress:
        head = struct.pack(hf, len(raw))
        if not b64:
            return head + raw
        if joint:
            return base64.b64encode(head + raw)
        return base64.b64encode(head) + base64.b64encode(raw)
    bs = 64
    blocks = [raw[i:i + bs] for i in range(0, len(raw), bs)] or [b""]
    comp = [zlib.compress(b) for b in blocks]
    last = len(blocks[-1]) if len(blocks[-1]) != bs else 0
    head = struct.pack(hf, len(blocks)) + struct.pack(hf, bs) + struct.pack(hf, last)
    sizes = b"".join(struct.pack(hf, len(c)) for c in comp)
    if not b64:
        return head + sizes + b"".join(comp)
    return base64.b64encode(head) + base64.b64encode(sizes) + base64.b64encode(b"".join(comp))


def _write_encoded(path, arrays, mode, header="UInt32", compress=False, joint=True, unstructured=False,
                   cells=None):
    """arrays: list of (section, name, np array, ncomp); mode: binary | raw | base64."""
    typ = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64", np.dtype(np.int64): "Int64",
           np.dtype(np.int32): "Int32", np.dtype(np.uint8): "UInt8"}
    kind = "UnstructuredGrid" if unstructured else "PolyData"
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    xml, app, off = [], b"", 0
    xml.append(f'<?xml version="1.0"?>\n<VTKFile type="{kind}" version="1.0" byte_order="LittleEndian" '
               f'header_type="{header}"{comp}>\n<{kind}>\n')
    npts = len([a for a in arrays if a[0] == "Points"][0][2]) // 3
    counts = f'NumberOfPoints="{npts}" ' + (f'NumberOfCells="{cells}"' if unstructured else 'NumberOfPolys="0"')
    xml.append(f"<Piece {counts}>\n")
    sections = []
    for sec, *_ in arrays:
        if sec not in sections:
            sections.append(sec)
    for sec in sections:
        attr = ' Normals="nn"' if sec == "CellData" else ""
        xml.append(f"<{sec}{attr}>\n")
        for s2, name, a, ncomp in arrays:
            if s2 != sec:
                continue
            payload = _enc_block(np.ascontiguousarray(a).tobytes(), header, compress, mode != "raw", joint)
            head = f'<DataArray type="{typ[a.dtype]}" Name="{name}" NumberOfComponents="{ncomp}"'
            if mode == "binary":
                xml.append(f'{head} format="binary">\n{payload.decode()}\n</DataArray>\n')
            else:
                xml.append(f'{head} format="appended" offset="{off}"/>\n')
                app += payload
                off += len(payload)
        xml.append(f"</{sec}>\n")
    xml.append(f"</Piece>\n</{kind}>\n")
    data = "".join(xml).encode()
    if mode != "binary":
        enc = "raw" if mode == "raw" else "base64"
        data += f'<AppendedData encoding="{enc}">\n_'.encode() + app + b"\n</AppendedData>\n"
    data += b"</VTKFile>\n"
    open(path, "wb").write(data)


@pytest.mark.parametrize("mode,header,compress,joint", [
    ("binary", "UInt32", False, True), ("binary", "UInt64", False, False), ("raw", "UInt64", False, True),
    ("base64", "UInt32", False, True), ("raw", "UInt32", True, True), ("binary", "UInt64", True, True)])
def test_point_cloud_reader_encodings(tmp_path, mode, header, compress, joint):
    p, n, r = _discs(40)
    soa = (r / (np.sqrt(3.0) / 2 * (1 + 1 / 32))).astype(np.float64)
    arrays = [("CellData", "nn", (n * 3.0).astype(np.float64).ravel(), 3), ("CellData", "sqrt-of-area", soa, 1),
              ("Points", "Points", p.astype(np.float64).ravel(), 3)]
    f = tmp_path / f"pc_{mode}_{header}_{compress}.vtp"
    _write_encoded(f, arrays, mode, header, compress, joint)
    try:
        p2, n2, r2 = vtk.read_point_cloud(str(f))
    except RtgError as e:
        if compress and "zlib" in str(e):
            pytest.skip("library built without zlib")
        raise
    np.testing.assert_array_equal(p2, p)
    # normals of length 3 are normalised (utils.hpp is_normalized / normalize)
    np.testing.assert_allclose(n2, n, rtol=0, atol=3e-7)
    # radius = sqrt-of-area * sqrt(3)/2 * (1 + 1/32) (vtp_point_cloud_reader.hpp:75-81)
    np.testing.assert_allclose(r2, (soa * np.sqrt(3.0) / 2 * (1 + 1 / 32)).astype(np.float32), rtol=1e-6)


def test_unstructured_triangles_skip_other_cells(tmp_path):
    v = RNG.random((8, 3)).astype(np.float32)
    conn = np.array([0, 1, 2, 3, 4, 5, 6, 1, 2, 7], np.int64)  # triangle, quad, triangle
    offs = np.array([3, 7, 10], np.int64)
    types = np.array([5, 9, 5], np.uint8)
    arrays = [("Points", "Points", v.ravel(), 3), ("Cells", "connectivity", conn, 1), ("Cells", "offsets", offs, 1),
              ("Cells", "types", types, 1)]
    f = tmp_path / "u.vtu"
    _write_encoded(f, arrays, "raw", "UInt64", False, unstructured=True, cells=3)
    v2, t2 = vtk.read_triangles(str(f))
    np.testing.assert_array_equal(v2, v)
    np.testing.assert_array_equal(t2, [[0, 1, 2], [1, 2, 7]])
    # an offset past the connectivity array is refused, not read
    g = tmp_path / "u_bad.vtu"
    arrays[2] = ("Cells", "offsets", np.array([3, 7, 13], np.int64), 1)
    _write_encoded(g, arrays, "raw", "UInt64", False, unstructured=True, cells=3)
    with pytest.raises(RtgError, match="offsets"):
        vtk.read_triangles(str(g))


def test_reader_errors(tmp_path):
    with pytest.raises(RtgError, match="cannot open"):
        vtk.read_point_cloud(str(tmp_path / "missing.vtp"))
    f = tmp_path / "nr.vtp"
    p, n, _ = _discs(3)
    _write_encoded(f, [("CellData", "nn", n.astype(np.float64).ravel(), 3),
                       ("Points", "Points", p.astype(np.float64).ravel(), 3)], "binary")
    with pytest.raises(RtgError, match="radius"):
        vtk.read_point_cloud(str(f))


def test_reader_rejects_damaged_data(tmp_path):
    """Sizes and offsets read from a file are checked against the file before
    anything is read or allocated: a damaged header is an error, not a read
    past the data or a huge allocation."""
    p, n, r = _discs(5)
    arrays = [("CellData", "nn", n.astype(np.float64).ravel(), 3), ("CellData", "radius", r.astype(np.float64), 1),
              ("Points", "Points", p.astype(np.float64).ravel(), 3)]
    good = tmp_path / "good.vtp"
    _write_encoded(good, arrays, "raw", "UInt64")
    vtk.read_point_cloud(str(good))  # the undamaged file reads
    data = good.read_bytes()
    at = data.index(b'encoding="raw">\n_') + len(b'encoding="raw">\n_')
    cases = {
        "huge array size": data[:at] + (1 << 60).to_bytes(8, "little") + data[at + 8:],
        "array size that wraps": data[:at] + ((1 << 64) - 1).to_bytes(8, "little") + data[at + 8:],
        "offset past the end": data.replace(b'offset="0"', b'offset="99999999"', 1),
    }
    _write_encoded(good, arrays, "base64", "UInt64")
    cases["base64 offset past the end"] = good.read_bytes().replace(b'offset="0"', b'offset="99999999"', 1)
    _write_encoded(good, arrays, "raw", "UInt64", compress=True)
    z = good.read_bytes()
    zat = z.index(b'encoding="raw">\n_') + len(b'encoding="raw">\n_')
    cases["huge block count"] = z[:zat] + (1 << 61).to_bytes(8, "little") + z[zat + 8:]
    for name, blob in cases.items():
        f = tmp_path / "bad.vtp"
        f.write_bytes(blob)
        with pytest.raises(RtgError, match="out of range|truncated|compressed"):
            vtk.read_point_cloud(str(f))


def test_segment_log_vtp_writer(rtg_lib, tmp_path):
    """rtg_write_vtp_segments (no GPU): one line cell per segment, two points
    each (origin, end), the cell arrays in record order."""
    import ctypes as C

    from rti_gb300 import _lib as L
    seg = np.zeros(3, dtype=L.SEGMENT_DTYPE)
    seg["ray"] = [7, 7, 9]
    seg["segment"] = [0, 1, 0]
    seg["kind"] = [L.RTG_SEG_HIT, L.RTG_SEG_ESCAPE, L.RTG_SEG_BOUNDARY]
    seg["org"] = [[0, 0, 1], [0.5, 0.5, 0], [1, 1, 1]]
    seg["end"] = [[0.5, 0.5, 0], [0.25, 0.75, 1], [2, 1, 1]]
    seg["primitive"] = [4, -1, -1]
    seg["weight"] = [1.0, 0.99, 1.0]
    f = tmp_path / "log.vtp"
    assert rtg_lib.rtg_write_vtp_segments(str(f).encode(), C.c_void_p(seg.ctypes.data), 3) == 0
    piece = ET.parse(f).getroot().find("PolyData/Piece")
    assert piece.get("NumberOfLines") == "3" and piece.get("NumberOfPoints") == "6"
    _, _, cells = _cell_arrays(f)
    assert cells["ray"][0] == "UInt64" and cells["kind"][0] == "Int32"
    np.testing.assert_array_equal(cells["ray"][2], [7, 7, 9])
    np.testing.assert_array_equal(cells["kind"][2], seg["kind"])
    np.testing.assert_array_equal(cells["primitive"][2], [4, -1, -1])
    np.testing.assert_allclose(cells["weight"][2], seg["weight"])
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=np.float64).reshape(-1, 3)
    np.testing.assert_allclose(pts[0::2], seg["org"])
    np.testing.assert_allclose(pts[1::2], seg["end"])
    lines = piece.find("Lines")
    conn = np.array(lines.findall("DataArray")[0].text.split(), dtype=np.int64)
    np.testing.assert_array_equal(conn, np.arange(6))
    assert rtg_lib.rtg_write_vtp_segments(None, None, 0) == L.RTG_ERR_INVALID_ARGUMENT


def _vtu(path, points, point_data=(), cell_data=(), cells=None):
    """A minimal ASCII UnstructuredGrid: vertex cells unless `cells` (lists of ids) is given."""
    def arr(name, a, ncomp):
        vals = " ".join(repr(float(x)) for x in np.asarray(a, np.float64).ravel())
        return (f'<DataArray type="Float64" Name="{name}" NumberOfComponents="{ncomp}" format="ascii">'
                f'{vals}</DataArray>')
    n = len(points)
    cells = cells if cells is not None else [[i] for i in range(n)]
    conn = " ".join(str(i) for c in cells for i in c)
    offs = " ".join(str(x) for x in np.cumsum([len(c) for c in cells]))
    types = " ".join("5" if len(c) == 3 else "1" for c in cells)
    pd = "".join(arr(nm, a, 1 if np.ndim(a) == 1 else 3) for nm, a in point_data)
    cd = "".join(arr(nm, a, 1 if np.ndim(a) == 1 else 3) for nm, a in cell_data)
    path.write_text(
        '<?xml version="1.0"?><VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian">'
        f'<UnstructuredGrid><Piece NumberOfPoints="{n}" NumberOfCells="{len(cells)}">'
        f'<PointData>{pd}</PointData><CellData>{cd}</CellData>'
        f'<Points>{arr("Points", points, 3)}</Points>'
        f'<Cells><DataArray type="Int64" Name="connectivity" format="ascii">{conn}</DataArray>'
        f'<DataArray type="Int64" Name="offsets" format="ascii">{offs}</DataArray>'
        f'<DataArray type="UInt8" Name="types" format="ascii">{types}</DataArray></Cells>'
        '</Piece></UnstructuredGrid></VTKFile>')


def test_vtu_point_cloud_readers(rtg_lib, tmp_path):
    """rti's io/christoph and io/xaver point readers: radius rules, z inversion
    (christoph), points with zero area / zero normal left out, normals normalised."""
    from rti_gb300 import _lib as L
    pts = np.array([[0.0, 0.0, 1.0], [1.0, 2.0, 3.0], [2.0, 0.5, -1.0], [3.0, 3.0, 3.0]])
    nrm = np.array([[0.0, 0.0, 2.0], [0.0, 0.0, 0.0], [0.6, 0.0, 0.8], [1.0, 0.0, 0.0]])
    area = np.array([0.04, 0.01, 0.09, 0.0])
    f = tmp_path / "christoph.vtu"
    _vtu(f, pts, point_data=[("area_around_vertex", area), ("normal_vector", nrm)])
    p, n, r = vtk.read_point_cloud_vtu(str(f), L.RTG_VTU_AREA)
    grow = np.sqrt(3.0) / 2 * 1.25
    keep = [0, 2]  # point 1 has the zero normal, point 3 zero area
    np.testing.assert_array_equal(p, (pts[keep] * [1, 1, -1]).astype(np.float32))
    np.testing.assert_allclose(n, [[0, 0, -1], [0.6, 0, -0.8]], atol=1e-7)
    np.testing.assert_allclose(r, np.sqrt(area[keep]) * grow, rtol=1e-6)
    # the christoph reader falls back to a gridSpacing cell array (still through the square root)
    g = tmp_path / "spacing.vtu"
    spacing = np.array([0.02, 0.02, 0.0, 0.05])
    _vtu(g, pts, point_data=[("normal_vector", nrm)], cell_data=[("gridSpacing", spacing)])
    _, _, r2 = vtk.read_point_cloud_vtu(str(g), L.RTG_VTU_AREA)
    np.testing.assert_allclose(r2, np.sqrt([0.02, 0.05]) * grow, rtol=1e-6)
    # xaver: gridSpacing itself, z kept
    p3, n3, r3 = vtk.read_point_cloud_vtu(str(g), L.RTG_VTU_SPACING)
    np.testing.assert_array_equal(p3, pts[[0, 3]].astype(np.float32))
    np.testing.assert_allclose(r3, np.array([0.02, 0.05]) * grow, rtol=1e-6)
    np.testing.assert_allclose(n3, [[0, 0, 1], [1, 0, 0]], atol=1e-7)
    with pytest.raises(RtgError, match="gridSpacing"):
        vtk.read_point_cloud_vtu(str(f), L.RTG_VTU_SPACING)


def test_vtu_triangle_reader(rtg_lib, tmp_path):
    """rti's io/christoph mesh reader: three-point cells with the second and
    third vertex swapped, mean vertex normals normalised, (0, 0, 1) where all
    three mean components are below 1e-5 (signed, as the reference)."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float64)
    vn = np.array([[0, 0, 2], [0, 0, 1], [0, 0, 1], [-1, 0, 0]], np.float64)
    cells = [[0, 1, 2], [1, 3, 2], [0, 3], [3, 3, 3]]
    f = tmp_path / "mesh.vtu"
    _vtu(f, v, point_data=[("normal_vector", vn)], cells=cells)
    vx, ix, nx = vtk.read_triangles_vtu(str(f))
    np.testing.assert_array_equal(vx, v.astype(np.float32))
    np.testing.assert_array_equal(ix, [[0, 2, 1], [1, 2, 3], [3, 3, 3]])
    np.testing.assert_allclose(nx[0], [0, 0, 1], atol=1e-7)
    m = (vn[1] + vn[3] + vn[2]) / 3
    np.testing.assert_allclose(nx[1], m / np.linalg.norm(m), atol=1e-6)
    np.testing.assert_allclose(nx[2], [0, 0, 1])  # mean (-1, 0, 0): every component below 1e-5
    # offsets past the connectivity array are refused, not read
    bad = tmp_path / "bad.vtu"
    bad.write_text(f.read_text().replace('Name="offsets" format="ascii">3 6 8 11<',
                                         'Name="offsets" format="ascii">3 6 8 14<'))
    assert bad.read_text() != f.read_text()
    with pytest.raises(RtgError, match="offsets"):
        vtk.read_triangles_vtu(str(bad))
