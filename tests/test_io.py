"""CPU checks of the reference-compatible file I/O in libpdfs (no GPU needed):
the reader against the golden input files, the writer against the
reference writer's format."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from pdfs_gb300 import _lib as L
from pdfs_gb300 import vti as VT

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vti")
CASES = {
    "sphere": (18, 16, 14, (1.0, 1.0, 1.0), (8.5, 7.0, 6.5), 4.2),
    "aniso": (15, 13, 20, (0.5, 0.7, 0.4), (3.6, 4.1, 3.9), 2.3),
}


def read(path):
    pf = L.Phi()
    s = L.load().pdfs_vti_read(path.encode(), C.byref(pf))
    return s, pf


@pytest.mark.parametrize("name", sorted(CASES))
def test_reader_parses_reference_input_layout(name):
    nx, ny, nz, sp, c, r = CASES[name]
    s, pf = read(os.path.join(GOLD, f"{name}_in.vti"))
    assert s == L.PDFS_OK
    try:
        assert (pf.x, pf.y, pf.z) == (nx, ny, nz)
        assert (pf.dx, pf.dy, pf.dz) == sp
        n = (nx + 2) * (ny + 2) * (nz + 2)
        loc = np.ctypeslib.as_array(pf.location, shape=(n,)).reshape(nz + 2, ny + 2, nx + 2)
        dist = np.ctypeslib.as_array(pf.distance, shape=(n,)).reshape(nz + 2, ny + 2, nx + 2)
        eloc, edist = VT.sphere_input(nx, ny, nz, sp, c, r)
        assert np.array_equal(loc[1:-1, 1:-1, 1:-1], eloc)
        assert dist[1:-1, 1:-1, 1:-1].tobytes() == edist.tobytes()
        # halo: border location -1, distance +inf (vti_parser.c:131-133,172-173)
        halo = np.ones(loc.shape, bool)
        halo[1:-1, 1:-1, 1:-1] = False
        assert (loc[halo] == -1).all() and np.isinf(dist[halo]).all()
    finally:
        L.load().pdfs_phi_free(C.byref(pf))


def test_reader_errors():
    s, _ = read("/nonexistent/file.vti")
    assert s == L.PDFS_ERR_IO
    import tempfile
    with tempfile.NamedTemporaryFile("w", suffix=".vti", delete=False) as f:
        f.write("<VTKFile>\n  no header here\n")
    try:
        s, _ = read(f.name)
        assert s == L.PDFS_ERR_IO
    finally:
        os.unlink(f.name)
    with tempfile.NamedTemporaryFile("w", suffix=".vti", delete=False) as f:
        # truncated data: header claims 2x2x2 interior nodes, only 3 values follow
        f.write('<?xml version="1.0"?>\n<VTKFile>\n    <ImageData WholeExtent="0 1 0 1 0 1" Spacing="1 1 1">\n'
                "a\nb\nc\n1 0 1\n")
    try:
        s, _ = read(f.name)
        assert s == L.PDFS_ERR_IO
    finally:
        os.unlink(f.name)


def python_writer(field, spacing):
    """The reference writer's byte format, restated in Python (file_writer.c:152-190)."""
    Z, Y, X = field.shape
    out = ['<?xml version="1.0"?>\n',
           '<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">\n',
           '\t<ImageData WholeExtent="0 %d 0 %d 0 %d" Origin="0 0 0" Spacing=" %f %f %f  ">\n'
           % (X - 1, Y - 1, Z - 1, *spacing),
           '\t\t<Piece Extent="0 %d 0 %d 0 %d">\n' % (X - 1, Y - 1, Z - 1),
           '\t\t\t<PointData Scalars="Distance Field">\n',
           '\t\t\t\t<DataArray type="Float32" Name="Distance Field" format="ascii">\n']
    for k in range(Z):
        for j in range(Y):
            out.append("".join("%f  " % v for v in field[k, j]) + "\n")
        out.append("\n")
    out += ['\t\t\t\t</DataArray>\n', '\t\t\t</PointData>\n', '\t\t\t<CellData>\n', '\t\t\t</CellData>\n',
            '\t\t</Piece>\n', '\t</ImageData>\n', '</VTKFile>\n']
    return "".join(out).encode()


def test_writer_matches_reference_format(tmp_path):
    rng = np.random.default_rng(4)
    nx, ny, nz = 7, 5, 4
    f = rng.uniform(-2, 50, size=(nz + 2, ny + 2, nx + 2))
    f[0, 0, 0] = math.inf
    f[1, 1, 1] = -1.0
    f[2, 2, 2] = 90000.0
    pf = L.Phi(nx, ny, nz, 0.5, 0.25, 1.0, None, f.ctypes.data_as(C.POINTER(C.c_double)), 1.0)
    out = tmp_path / "o.vti"
    assert L.load().pdfs_vti_write(str(out).encode(), C.byref(pf)) == L.PDFS_OK
    assert out.read_bytes() == python_writer(f, (0.5, 0.25, 1.0))
    ext, sp, vals = VT.read_output(str(out))
    assert ext == (nx + 2, ny + 2, nz + 2) and sp == (0.5, 0.25, 1.0)
    assert np.allclose(vals, f, atol=5e-7)


def test_reference_output_fixture_is_in_writer_format():
    """The golden reference outputs round-trip through the Python restatement."""
    for name in CASES:
        raw = open(os.path.join(GOLD, f"{name}_ref_distfield.vti"), "rb").read()
        ext, sp, vals = VT.read_output(os.path.join(GOLD, f"{name}_ref_distfield.vti"))
        assert python_writer(vals, sp) == raw
