"""VTI files in the reference's formats (Python side, for tests and users).

write_input() produces the input layout that the reference's reader
(single_gpu_cuda/src/vti_parser.c:85-180) and pdfs_vti_read() accept: a
header whose third line carries WholeExtent and Spacing, the interior
`location` ints starting on line 7, one separator line, the interior
`distance` values.  read_output() parses the writer's output
(single_gpu_cuda/src/file_writer.c:152-190): the whole halo-padded grid.
"""
from __future__ import annotations

import re

import numpy as np


def write_input(path, location, distance, spacing):
    """location, distance: interior arrays shaped (nz, ny, nx)."""
    location = np.asarray(location)
    distance = np.asarray(distance, dtype=np.float64)
    nz, ny, nx = distance.shape
    dx, dy, dz = spacing
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n')
        f.write('<VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">\n')
        f.write(f'    <ImageData WholeExtent="0 {nx - 1} 0 {ny - 1} 0 {nz - 1}" Spacing="{dx!r} {dy!r} {dz!r}">\n')
        f.write(f'      <Piece Extent="0 {nx - 1} 0 {ny - 1} 0 {nz - 1}">\n')
        f.write('        <PointData>\n')
        f.write('          <DataArray type="Int32" Name="location" format="ascii">\n')
        for plane in location.reshape(nz, ny, nx):
            for row in plane:
                f.write(" ".join(str(int(v)) for v in row) + "\n")
        f.write('          </DataArray>\n')
        f.write('          <DataArray type="Float64" Name="distance" format="ascii">\n')
        for plane in distance:
            for row in plane:
                f.write(" ".join(repr(float(v)) for v in row) + "\n")
        f.write('          </DataArray>\n')
        f.write('        </PointData>\n')
        f.write('      </Piece>\n')
        f.write('    </ImageData>\n')
        f.write('</VTKFile>\n')


def read_output(path):
    """Returns (extent (X, Y, Z) of the halo-padded grid, spacing, values
    shaped (Z, Y, X)) from a file in the reference writer's format."""
    txt = open(path).read()
    m = re.search(r'WholeExtent="0 (\d+) 0 (\d+) 0 (\d+)"', txt)
    s = re.search(r'Spacing="\s*([^"]+)"', txt)
    X, Y, Z = (int(v) + 1 for v in m.groups())
    spacing = tuple(float(v) for v in s.group(1).split())
    body = txt.split('format="ascii">\n', 1)[1].split("</DataArray>", 1)[0]
    vals = np.array([float(v) for v in body.split()])
    return (X, Y, Z), spacing, vals.reshape(Z, Y, X)


def sphere_input(nx, ny, nz, spacing, centre, radius, band=1.0):
    """A sphere interface in the reference's input convention: location 1
    inside the sphere, 0 outside; distance = |r - R| for nodes within `band`
    spacings of the surface, 0 (unknown) elsewhere."""
    h = max(spacing)
    z, y, x = np.meshgrid(np.arange(nz) * spacing[2], np.arange(ny) * spacing[1], np.arange(nx) * spacing[0],
                          indexing="ij")
    r = np.sqrt((x - centre[0]) ** 2 + (y - centre[1]) ** 2 + (z - centre[2]) ** 2)
    loc = (r < radius).astype(np.int32)
    d = np.abs(r - radius)
    dist = np.where(d <= band * h, d, 0.0)
    return loc, dist
