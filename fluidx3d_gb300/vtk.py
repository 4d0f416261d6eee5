"""Binary legacy VTK files in the reference's format (host side).

  * fields: src/lbm.hpp:298-340 ``Memory_Container::write_vtk`` -- STRUCTURED_POINTS, one point per
    cell (x fastest), values big-endian, the components of a 3-vector interleaved per point, FP32
    values multiplied by the unit-conversion factor;
  * meshes: src/lbm.cpp:1094-1129 ``LBM::write_mesh_to_vtk`` -- POLYDATA, three points per
    triangle, shifted by the box centre and scaled by the cell size;
  * file names: src/lbm.cpp:85-92 ``default_filename`` -- ``<path><name>-<t, 9 digits>.vtk``.

The device-side writer of a field is ``lbm_write_vtk`` in the C-ABI (packing on the GPU); the
host-side writer here produces the same bytes from a host copy.
"""
from __future__ import annotations

import os
import sys

import numpy as np

f32 = np.float32


def export_folder() -> str:
    """The reference writes to <executable's folder>/export/ by default; here the folder of the
    running script."""
    return os.path.join(os.path.dirname(os.path.abspath(sys.argv[0] or ".")), "export") + os.sep


def default_filename(path: str, name: str, extension: str, t: int) -> str:
    time = ("00000000" + str(int(t)))[-9:]
    base = (name or "file") + "-" + time
    return (path if path else export_folder()) + create_file_extension(base, extension)


def create_file_extension(filename: str, extension: str) -> str:
    """src/utilities.hpp:4205-4207: replace the extension after the last '.' (or append one)."""
    dot = filename.rfind(".")
    stem = filename[:dot] if dot != -1 else filename
    return stem + ("" if extension.startswith(".") else ".") + extension


def _create_folder(filename: str) -> None:
    slash = filename.rfind("/")
    if slash > 0:
        os.makedirs(filename[:slash], exist_ok=True)


def field_header(filename: str, shape, spacing: float, vtk_type: str, dims: int) -> bytes:
    Nx, Ny, Nz = (int(v) for v in shape)
    s = f32(spacing)
    origin = [s * (f32(0.5) - f32(0.5) * f32(n)) for n in (Nx, Ny, Nz)]
    title = filename[filename.rfind("/") + 1:]
    return ("# vtk DataFile Version 3.0\nFluidX3D " + title + "\nBINARY\nDATASET STRUCTURED_POINTS\n"
            f"DIMENSIONS {Nx} {Ny} {Nz}\n"
            f"ORIGIN {float(origin[0]):f} {float(origin[1]):f} {float(origin[2]):f}\n"
            f"SPACING {float(s):f} {float(s):f} {float(s):f}\n"
            f"POINT_DATA {Nx * Ny * Nz}\n"
            f"SCALARS data {vtk_type} {dims}\nLOOKUP_TABLE default\n").encode()


def write_field_vtk(filename: str, data: np.ndarray, shape, dims: int, spacing: float = 1.0, scale: float = 1.0) -> str:
    """Writes a host field (SoA, ``dims`` blocks of N) as the reference's binary .vtk file."""
    filename = create_file_extension(filename, ".vtk")
    N = int(shape[0]) * int(shape[1]) * int(shape[2])
    data = np.asarray(data)
    if data.size != N * dims:
        raise ValueError(f"field has {data.size} values, expected {N * dims}")
    if data.dtype == np.uint8:
        vtk_type, body = "unsigned_char", data.reshape(dims, N).T.tobytes()
    elif data.dtype == np.float32:
        scaled = f32(scale) * data if scale != 1.0 else data
        vtk_type, body = "float", np.ascontiguousarray(scaled.reshape(dims, N).T).astype(">f4").tobytes()
    else:
        raise TypeError(f"unsupported field type {data.dtype}")
    _create_folder(filename)
    with open(filename, "wb") as fh:
        fh.write(field_header(filename, shape, spacing, vtk_type, dims))
        fh.write(body)
    return filename


def write_mesh_vtk(filename: str, mesh, center, spacing: float = 1.0) -> str:
    """Writes a triangle mesh as the reference's binary POLYDATA .vtk file: vertex k of triangle i
    is point 3i+k at spacing*(p - center)."""
    filename = create_file_extension(filename, ".vtk")
    T = int(mesh.triangle_number)
    c = np.asarray(center, f32)
    s = f32(spacing)
    pts = np.empty((T, 3, 3), f32)
    for k, p in enumerate((mesh.p0, mesh.p1, mesh.p2)):
        pts[:, k, :] = s * (np.asarray(p, f32) - c)
    tri = np.empty((T, 4), np.int32)
    tri[:, 0] = 3
    tri[:, 1] = 3 * np.arange(T)
    tri[:, 2] = tri[:, 1] + 1
    tri[:, 3] = tri[:, 1] + 2
    title = filename[filename.rfind("/") + 1:]
    _create_folder(filename)
    with open(filename, "wb") as fh:
        fh.write(f"# vtk DataFile Version 3.0\nFluidX3D {title}\nBINARY\nDATASET POLYDATA\nPOINTS {3 * T} float\n".encode())
        fh.write(pts.astype(">f4").tobytes())
        fh.write(f"POLYGONS {T} {4 * T}\n".encode())
        fh.write(tri.astype(">i4").tobytes())
    return filename


def read_vtk(filename: str):
    """Reads back a STRUCTURED_POINTS file written above: (header dict, data as SoA numpy array)."""
    with open(filename, "rb") as fh:
        raw = fh.read()
    lines, pos = [], 0
    while len(lines) < 10:
        end = raw.index(b"\n", pos)
        lines.append(raw[pos:end].decode())
        pos = end + 1
    hdr = {"title": lines[1], "dimensions": tuple(int(v) for v in lines[4].split()[1:]),
           "origin": tuple(float(v) for v in lines[5].split()[1:]), "spacing": tuple(float(v) for v in lines[6].split()[1:]),
           "points": int(lines[7].split()[1]), "type": lines[8].split()[2], "dims": int(lines[8].split()[3])}
    dt = np.dtype(">f4") if hdr["type"] == "float" else np.dtype(np.uint8)
    vals = np.frombuffer(raw, dtype=dt, offset=pos)
    return hdr, np.ascontiguousarray(vals.reshape(hdr["points"], hdr["dims"]).T).reshape(-1).astype(dt.newbyteorder("="))
