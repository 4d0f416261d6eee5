"""Host-side checks that need no GPU: the C-ABI library loads and exports every symbol the header
declares, the Python binding covers them, and the host logic (relaxation-rate literal, byte
accounting, set-ups, meshes, error reporting without a device) behaves as the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
from fluidx3d_gb300 import _capi as C, setups as S, mesh as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "lbm_capi.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(solver_lib):
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(solver_lib, n), n
    assert set(names) == set(C.SIGNATURES), set(names) ^ set(C.SIGNATURES)


def test_relaxation_rate_is_the_reference_literal(solver_lib):
    for nu in (1.0 / 30.0, 0.048, 1e-4, 1.0, 0.02, 0.0123456):
        assert C.relaxation_rate(nu) == oracle.kernel_w(nu)
    # tau = 0.6: 1/tau printed "%f" -> 1.666667
    assert C.relaxation_rate(1.0 / 30.0) == np.float32(1.666667)


def test_bandwidth_accounting_matches_reference(solver_lib):
    def cfg(q, st, ext=0):
        return C.LBMConfig(8, 8, 8, q, 0, st, ext, -1, 0.1, 0, 0, 0)
    L = solver_lib
    assert L.lbm_bandwidth_bytes_per_cell(ctypes.byref(cfg(19, C.FP32))) == 153
    assert L.lbm_bandwidth_bytes_per_cell(ctypes.byref(cfg(19, C.FP16S))) == 77
    assert L.lbm_bandwidth_bytes_per_cell(ctypes.byref(cfg(19, C.FP16C))) == 77
    assert L.lbm_bandwidth_bytes_per_cell(ctypes.byref(cfg(27, C.FP32))) == 217
    assert L.lbm_bandwidth_bytes_per_cell(ctypes.byref(cfg(27, C.FP16S))) == 109
    assert L.lbm_bandwidth_bytes_per_cell(ctypes.byref(cfg(19, C.FP32, C.EXT_FORCE_FIELD))) == 165
    assert L.lbm_bytes_per_cell_device(ctypes.byref(cfg(19, C.FP32))) == 93
    assert L.lbm_bytes_per_cell_device(ctypes.byref(cfg(19, C.FP16S))) == 55


def test_invalid_configs_are_errors_not_exits(solver_lib):
    from fluidx3d_gb300 import LBM, LBMError
    for kwargs, status in [(dict(Nx=0, Ny=4, Nz=4, nu=0.1), 1), (dict(Nx=4, Ny=4, Nz=4, nu=0.0), 1), (dict(Nx=4, Ny=4, Nz=4, nu=-1.0), 1),
                           (dict(Nx=4, Ny=4, Nz=4, nu=0.1, fx=1e-5), 1)]:
        with pytest.raises(LBMError) as e:
            LBM(**kwargs)
        assert e.value.status in (status, 6)
    with pytest.raises(ValueError):
        LBM(4, 4, 4, 0.1, extensions=("surface",))


def test_taylor_green_initial_state():
    c = S.taylor_green(64, 64, 64)
    N = 64 ** 3
    ux, uy, uz = c["u"][:N], c["u"][N:2 * N], c["u"][2 * N:]
    assert abs(ux.max() - 0.05) < 1e-3 and np.all(uz == 0)
    # divergence-free and rho = 1 + 3 u0^2/16 (...)(...) averages to 1
    assert abs(float(np.mean(c["rho"].astype(np.float64))) - 1.0) < 1e-7
    assert np.allclose(ux.reshape(64, 64, 64)[:, :, ::-1][:, :, :], -ux.reshape(64, 64, 64)[:, :, :], atol=1e-7)


def test_sphere_channel_geometry():
    c = S.sphere_channel(64, 32, 32, radius=6.0, center=(16, 16, 16))
    f = c["flags"].reshape(32, 32, 64)
    assert np.all(f[0, :, :] == S.TYPE_S) and np.all(f[:, 0, :] == S.TYPE_S)
    assert np.all(f[5:-5, 5:-5, 0] == S.TYPE_E) and np.all(f[5:-5, 5:-5, -1] == S.TYPE_E)
    n_sphere = int(np.sum(f == (S.TYPE_S | S.TYPE_X)))
    assert abs(n_sphere - 4.0 / 3.0 * np.pi * 6 ** 3) / n_sphere < 0.1


def test_mesh_stl_roundtrip_and_closed_ellipsoid(tmp_path):
    m = M.ellipsoid_mesh((10, 11, 12), (5, 4, 3), n_theta=12, n_phi=24, noise_amplitude=0.5, seed=1)
    # closed, outward oriented: divergence theorem volume close to the ellipsoid's
    vol = np.sum(np.einsum("ij,ij->i", m.p0 - m.center, np.cross(m.p1 - m.center, m.p2 - m.center))) / 6.0
    assert abs(vol - 4.0 / 3.0 * np.pi * 60) / (4.0 / 3.0 * np.pi * 60) < 0.15
    p = tmp_path / "e.stl"
    M.write_stl(str(p), m)
    r = M.read_stl(str(p), size=-1.0, reposition=False)
    assert np.array_equal(r.p0, m.p0) and np.array_equal(r.p2, m.p2)
    assert r.triangle_number == 2 * 24 * 11
