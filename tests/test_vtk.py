"""Host-side I/O around the solver path: the VTK format of the reference's field and mesh export
(src/lbm.hpp:298-340, src/lbm.cpp:1094-1129), its file names (src/lbm.cpp:85-92), unit conversion
(src/units.hpp) and the binary STL reader (src/utilities.hpp:4530-4581). CPU only; the GPU writer
is compared with these in test_vtk_gpu.py."""
import struct

import numpy as np
import pytest

from fluidx3d_gb300 import vtk, Units
from fluidx3d_gb300.mesh import Mesh, read_stl, write_stl


def test_header_is_the_references():
    """Header lines as src/lbm.hpp:310-317 builds them (std::to_string of floats: "%f")."""
    h = vtk.field_header("out/dir/u-000000100.vtk", (40, 24, 20), 0.5, "float", 3).decode()
    assert h == ("# vtk DataFile Version 3.0\nFluidX3D u-000000100.vtk\nBINARY\nDATASET STRUCTURED_POINTS\n"
                 "DIMENSIONS 40 24 20\nORIGIN -9.750000 -5.750000 -4.750000\nSPACING 0.500000 0.500000 0.500000\n"
                 "POINT_DATA 19200\nSCALARS data float 3\nLOOKUP_TABLE default\n")


def test_field_round_trip_big_endian_interleaved(tmp_path):
    shape = (5, 4, 3)
    N = 60
    rng = np.random.default_rng(0)
    u = rng.normal(size=3 * N).astype(np.float32)
    fn = vtk.write_field_vtk(str(tmp_path / "u-000000007.vtk"), u, shape, 3, spacing=2.0, scale=3.0)
    raw = open(fn, "rb").read()
    body = raw[raw.index(b"LOOKUP_TABLE default\n") + len("LOOKUP_TABLE default\n"):]
    assert len(body) == 12 * N
    # point 1, component y, big-endian
    assert struct.unpack(">f", body[12 + 4:12 + 8])[0] == np.float32(3.0) * u[N + 1]
    hdr, back = vtk.read_vtk(fn)
    assert hdr["dimensions"] == shape and hdr["dims"] == 3 and hdr["type"] == "float" and hdr["spacing"] == (2.0, 2.0, 2.0)
    assert np.array_equal(back, np.float32(3.0) * u)
    flags = rng.integers(0, 256, N).astype(np.uint8)
    fn = vtk.write_field_vtk(str(tmp_path / "flags"), flags, shape, 1)
    assert fn.endswith("flags.vtk")
    hdr, back = vtk.read_vtk(fn)
    assert hdr["type"] == "unsigned_char" and np.array_equal(back, flags)


def test_file_names():
    assert vtk.default_filename("out/", "rho", ".vtk", 1234) == "out/rho-000001234.vtk"
    assert vtk.default_filename("out/", "", "vtk", 7) == "out/file-000000007.vtk"
    assert vtk.default_filename("", "u", ".vtk", 0).endswith("export/u-000000000.vtk")
    assert vtk.default_filename("a/", "u", ".vtk", 12345678901) == "a/u-345678901.vtk"  # 9 digits, as the reference cuts
    assert vtk.create_file_extension("x/y.stl", ".vtk") == "x/y.vtk"


def test_mesh_polydata(tmp_path):
    p0 = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]], np.float32)
    m = Mesh(p0, p0 + 1.0, p0 + np.float32([0.0, 2.0, 0.0]))
    fn = vtk.write_mesh_vtk(str(tmp_path / "mesh-000000000.vtk"), m, center=(0.5, 1.5, 2.5), spacing=2.0)
    raw = open(fn, "rb").read()
    head = b"# vtk DataFile Version 3.0\nFluidX3D mesh-000000000.vtk\nBINARY\nDATASET POLYDATA\nPOINTS 6 float\n"
    assert raw.startswith(head)
    pts = np.frombuffer(raw[len(head):len(head) + 72], ">f4").reshape(6, 3)
    assert np.array_equal(pts[0], np.float32(2.0) * (p0[0] - np.float32([0.5, 1.5, 2.5])))
    tail = raw[len(head) + 72:]
    assert tail.startswith(b"POLYGONS 2 8\n")
    assert np.array_equal(np.frombuffer(tail[len(b"POLYGONS 2 8\n"):], ">i4"), [3, 0, 1, 2, 3, 3, 4, 5])


def test_units_follow_the_reference():
    u = Units()
    assert u.si_u(0.05) == np.float32(0.05)  # identity by default
    u.set_m_kg_s(38.0, 0.05, 1.0, 0.2, 1.5, 1000.0)
    f = np.float32
    m = f(f(0.2) / f(38.0))
    kg = f(f(f(1000.0) / f(1.0)) * f(f(m * m) * m))
    s = f(f(f(0.05) / f(1.5)) * m)
    assert (u.unit_m, u.unit_kg, u.unit_s) == (m, kg, s)
    assert u.si_u(0.05) == f(f(f(0.05) * m) / s)
    assert abs(float(u.si_u(0.05)) - 1.5) < 1e-6
    assert abs(float(u.si_rho(1.0)) - 1000.0) < 1e-2
    assert abs(float(u.x(0.2)) - 38.0) < 1e-5
    assert u.t(u.si_t(1000)) == 1000
    with pytest.raises(TypeError):
        u.set_m_kg_s(1.0, 2.0)


def test_stl_reader_rescales_rotates_and_recentres(tmp_path):
    """read_stl_raw: rotate, fit the longest side to `size`, centre on `center`; reposition=False
    keeps the file coordinates (scaled by |scale|)."""
    rng = np.random.default_rng(3)
    p = rng.uniform(-3.0, 5.0, (3, 40, 3)).astype(np.float32)
    fn = str(tmp_path / "part.stl")
    write_stl(fn, Mesh(p[0], p[1], p[2]))
    R = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    m = read_stl(fn, box_size=(40, 24, 20), center=(19.5, 11.5, 9.5), rotation=R, size=16.0)
    assert m.triangle_number == 40
    ext = m.pmax - m.pmin
    assert abs(float(ext.max()) - 16.0) < 1e-4
    assert np.allclose(0.5 * (m.pmin + m.pmax), (19.5, 11.5, 9.5), atol=1e-4)
    # rotation by +90 degrees about z: x' = -y
    r0 = np.stack([-p[0][:, 1], p[0][:, 0], p[0][:, 2]], axis=1)
    d = m.p0 - m.p0[0]
    d_ref = (r0 - r0[0]) * (m.p0[1, 2] - m.p0[0, 2]) / (r0[1, 2] - r0[0, 2])
    assert np.allclose(d, d_ref, atol=1e-4)
    raw = read_stl(fn, reposition=False, size=-1.0)
    assert np.array_equal(raw.p1, p[1])
    with open(fn, "r+b") as fh:
        fh.truncate(84 + 50 * 39)
    with pytest.raises(ValueError):
        read_stl(fn)
