"""The CPU oracle against the golden fixtures produced by the reference's own kernels.

The fixtures (tests/golden/, made by tests/golden/make_golden.py from the reference's OpenCL C
kernel text compiled for the CPU) pin the oracle: it must reproduce them bit for bit.
"""
import hashlib
import os

import numpy as np
import pytest

import oracle
import lbm_cases as LC


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_oracle(case, precision="f32"):
    o = oracle.Oracle(*case.shape, q=case.q, collision=case.collision, storage=case.storage, extensions=case.extensions,
                      nu=case.nu, precision=precision)
    f = case.fields()
    o.rho[:], o.u[:], o.flags[:], o.F[:] = f["rho"], f["u"], f["flags"], f["F"]
    o.initialize()
    o.run(case.steps, *case.force)
    case.settle_fields(o)
    if "ff" in case.extensions:
        o.update_force_field()
    return o


@pytest.mark.parametrize("case", LC.CASES, ids=[c.name for c in LC.CASES])
def test_oracle_matches_reference_fixture(case, golden_dir):
    g = np.load(os.path.join(golden_dir, f"lbm_{case.name}.npz"))
    o = run_oracle(case)
    assert np.array_equal(o.rho, g["rho"])
    assert np.array_equal(o.u, g["u"])
    if "ff" in case.extensions:
        assert np.array_equal(o.F, g["F"])
    if "mb" in case.extensions:
        assert np.array_equal(o.flags, g["flags"])
        assert np.count_nonzero((o.flags & 3) == 3) > 0  # cells next to the moving walls are marked
    assert sha(o.fi) == str(g["fi_sha256"])


def test_oracle_taylor_green_64_matches_reference(golden_dir):
    """Config-1 workload (64^3 TGV, SRT FP32, tau=0.6, 1000 steps): bit-identical to the reference."""
    g = np.load(os.path.join(golden_dir, "tgv64.npz"))
    o = run_oracle(LC.TGV64)
    assert sha(o.rho) == str(g["rho_sha256"])
    assert sha(o.u) == str(g["u_sha256"])
    assert sha(o.fi) == str(g["fi_sha256"])
    n = 32 + (32 + 32 * 64) * 64
    assert o.u[n] == g["ux_center"]


def test_oracle_voxelization_matches_reference(golden_dir):
    g = np.load(os.path.join(golden_dir, "voxel.npz"))
    shape, mesh = LC.voxel_mesh_case()
    bbu, direction = LC.bbu_for(mesh)
    assert direction == int(g["direction"]) and np.array_equal(bbu.view(np.uint32), g["bbu"].view(np.uint32))
    o = oracle.Oracle(*shape, q=19, nu=0.1)
    o.voxelize_mesh(direction, 0x01, mesh.p0.reshape(-1), mesh.p1.reshape(-1), mesh.p2.reshape(-1), bbu, 1)
    assert np.array_equal(o.flags, g["flags"])
    assert int(np.sum(o.flags == 1)) == int(g["solid_cells"]) > 1000


def test_fp64_oracle_tracks_fp32():
    """The FP64 restatement is the same scheme: it stays within FP32 rounding of the FP32 run."""
    case = LC.CASE_BY_NAME["d3q19_trt_fp32_channel_eq_ff_vf"]
    a, b = run_oracle(case, "f32"), run_oracle(case, "f64")
    assert np.max(np.abs(a.u - b.u)) / np.max(np.abs(b.u)) < 1e-5
    assert np.max(np.abs(a.rho - b.rho)) < 1e-5


def test_oracle_update_moving_boundaries_marks_like_initialize():
    """update_moving_boundaries after initialize changes nothing (same marking, TYPE_T aside), and
    stopping the lid clears every TYPE_MS mark."""
    case = LC.CASE_BY_NAME["d3q19_srt_fp32_cavity_mb"]
    o = oracle.Oracle(*case.shape, q=case.q, collision=case.collision, storage=case.storage, extensions=case.extensions, nu=case.nu)
    f = case.fields()
    o.rho[:], o.u[:], o.flags[:] = f["rho"], f["u"], f["flags"]
    o.initialize()
    marked = o.flags.copy()
    o.update_moving_boundaries()
    assert np.array_equal(o.flags, marked)
    o.u[:] = 0.0
    o.update_moving_boundaries()
    assert np.count_nonzero((o.flags & 3) == 3) == 0
    assert np.array_equal(o.flags, f["flags"])
