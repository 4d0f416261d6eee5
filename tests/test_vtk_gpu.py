"""VTK export straight from the GPU (lbm_write_vtk: scaling, interleaving and byte order on the
device, chunked and overlapped with the file writes) against the host-side writer of the same field,
from Python and from a C++ setup over fluidx3d_gb300/host/lbm.hpp; and the C++ STL reader and mesh
export against the Python ones."""
import os
import subprocess

import numpy as np
import pytest

from fluidx3d_gb300 import LBM, LBMError, units, vtk
from fluidx3d_gb300.mesh import read_stl, write_stl, ellipsoid_mesh
from fluidx3d_gb300 import setups as S

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def same_bytes(a, b):
    with open(a, "rb") as fa, open(b, "rb") as fb:
        return fa.read() == fb.read()


def test_device_writer_equals_host_writer(gpu, tmp_path):
    """rho, u, flags and F of a sphere channel after 10 steps, lattice and SI units; u is 17.4M
    values, so the device writer goes through two chunks."""
    Nx, Ny, Nz = 190, 180, 170
    f = S.sphere_channel(Nx, Ny, Nz, u_in=0.05, radius=20.0, center=(60.0, 90.0, 85.0))
    saved = (units.unit_m, units.unit_kg, units.unit_s)
    try:
        with LBM(Nx, Ny, Nz, 0.05, extensions=("eq",)) as lbm:
            lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:] = f["rho"], f["u"], f["flags"]
            lbm.run(10)
            lbm.update_force_field()
            for si in (False, True):
                if si:
                    units.set_m_kg_s(168.0, 0.05, 1.0, 0.5, 2.0, 1000.0)
                for field in (lbm.rho, lbm.u, lbm.flags, lbm.F):
                    dev = field.write_device_to_vtk(str(tmp_path / f"dev{si}") + "/", si)
                    field.read_from_device()
                    host = field.write_host_to_vtk(str(tmp_path / f"host{si}") + "/", si)
                    assert dev.endswith(f"{field.name}-000000010.vtk")
                    assert os.path.getsize(dev) > field.data.nbytes
                    assert same_bytes(dev, host), (field.name, si)
            hdr, u = vtk.read_vtk(str(tmp_path / "devFalse" / "u-000000010.vtk"))
            assert hdr["dims"] == 3 and np.array_equal(u, lbm.u.data)
    finally:
        units.set_m_kg_s(*saved)


def test_device_writer_refusals(gpu, tmp_path):
    with LBM(8, 8, 8, 0.05) as lbm:
        lbm.run(1)
        with pytest.raises(LBMError) as e:  # F does not exist yet
            lbm.F.write_device_to_vtk(str(tmp_path) + "/")
        assert e.value.status == 5
        blocker = tmp_path / "blocker"
        blocker.write_text("")
        with pytest.raises(LBMError) as e:  # the folder is a file
            lbm.rho.write_device_to_vtk(str(blocker) + "/")
        assert e.value.status == 7


def test_cpp_setup_vtk_and_stl(gpu, solver_lib, tmp_path):
    """The C++ host layer's device and host writers give identical files; its STL reader and mesh
    export give the bytes the Python ones give."""
    from fluidx3d_gb300 import build
    exe = tmp_path / "vtk_setup"
    libdir = os.path.dirname(build.LIB_PATH)
    # without contraction, so the host layer's FP32 arithmetic is the Python mirror's on every machine
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-DVOLUME_FORCE", "-DFORCE_FIELD", "-DEQUILIBRIUM_BOUNDARIES",
                    "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "fluidx3d_gb300", "host"),
                    os.path.join(ROOT, "tests", "cpp", "vtk_export_setup.cpp"), "-L", libdir, "-lfluidx3d_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    mesh = ellipsoid_mesh(center=(0.0, 0.0, 0.0), semi_axes=(3.0, 2.0, 1.5), n_theta=8, n_phi=16, seed=1)
    stl = str(tmp_path / "part.stl")
    write_stl(stl, mesh)
    out = tmp_path / "out"
    res = subprocess.run([str(exe), str(out), stl], check=True, capture_output=True, text=True).stdout.split()
    assert res[0:2] == ["t", "10"]
    for name in ("rho", "u", "flags", "F"):
        assert same_bytes(out / "device" / f"{name}-000000010.vtk", out / "host" / f"{name}-000000010.vtk"), name
    for name in ("u", "F"):
        assert same_bytes(out / "si" / "device" / f"{name}-000000010.vtk", out / "si" / "host" / f"{name}-000000010.vtk"), name
    hdr, _ = vtk.read_vtk(str(out / "si" / "device" / "u-000000010.vtk"))
    assert abs(hdr["spacing"][0] - 0.2 / 38.0) < 1e-6
    R = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    m = read_stl(stl, box_size=(40, 24, 20), center=(19.5, 11.5, 9.5), rotation=R, size=16.0)
    assert [np.float32(v) for v in res[5:8] + res[9:12]] == [*m.pmin, *m.pmax]
    py = vtk.write_mesh_vtk(str(tmp_path / "py" / "mesh-000000010.vtk"), m, center=(19.5, 11.5, 9.5), spacing=1.0)
    assert same_bytes(out / "mesh-000000010.vtk", py)
