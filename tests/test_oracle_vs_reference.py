"""The CPU oracle against the reference's kernels compiled for the CPU, on randomised inputs.

Runs only where the reference-kernel harness could be built (oracle/_ref/, which needs the
reference's kernel text); elsewhere the golden fixtures carry the same check.
"""
import numpy as np
import pytest

import oracle
from oracle.ref_harness import build_ref


def _harness(variant):
    try:
        built = build_ref.build_all([variant], jobs=1)
    except Exception as e:  # noqa: BLE001
        pytest.skip(f"reference harness unavailable: {e}")
    if not built:
        pytest.skip("reference kernel text unavailable")


VARIANTS = [(19, "srt", "fp32", ("eq", "ff", "vf")), (19, "trt", "fp16s", ("eq", "ff", "vf")), (19, "srt", "fp16c", ("eq",)),
            (27, "trt", "fp32", ("eq", "ff", "vf")), (27, "srt", "fp16s", ()),
            (19, "srt", "fp32", ("sg",)), (19, "trt", "fp16s", ("eq", "sg")), (27, "trt", "fp32", ("eq", "ff", "sg", "vf")),
            (19, "srt", "fp32", ("mb",)), (19, "trt", "fp16s", ("mb",)), (19, "trt", "fp16c", ("mb", "sg")),
            (27, "trt", "fp32", ("eq", "ff", "mb", "vf")),
            (19, "srt", "fp32", ("uf",)), (19, "trt", "fp16s", ("eq", "ff", "uf", "vf")), (27, "trt", "fp16c", ("eq", "mb", "uf"))]


@pytest.mark.parametrize("variant", VARIANTS, ids=["_".join([str(v[0]), v[1], v[2], *v[3]]) for v in VARIANTS])
def test_random_flags_and_fields(variant):
    """Random fluid/solid/equilibrium cells, random rho/u/F, odd box: every kernel bit-identical.
    MOVING_BOUNDARIES: solid cells keep their random velocities (moving walls); stale TYPE_MS and
    TYPE_T cells are in the mix, and halfway the solids' velocities change and
    update_moving_boundaries re-marks the cells next to them."""
    _harness(variant)
    q, col, st, ext = variant
    mb = "mb" in ext
    Nx, Ny, Nz = 13, 9, 7
    N = Nx * Ny * Nz
    rng = np.random.default_rng(42)
    mix = [0, 0, 0, 0, 0x01, 0x02 if "eq" in ext else 0, 0x41] + ([0x03, 0x04, 0x01] if mb else [])
    flags = rng.choice(np.array(mix, np.uint8), N)
    rho = (1.0 + rng.normal(0, 0.01, N)).astype(np.float32)
    u = rng.normal(0, 0.03, 3 * N).astype(np.float32)
    F = rng.normal(0, 2e-4, 3 * N).astype(np.float32)
    runs = []
    for cls in (oracle.RefHarness, oracle.Oracle):
        m = cls(Nx, Ny, Nz, q=q, collision=col, storage=st, extensions=ext, nu=0.02)
        m.rho[:], m.u[:], m.flags[:], m.F[:] = rho, u, flags, F
        m.initialize()
        states = [m.fi.copy()]
        fx = 3e-5 if "vf" in ext else 0.0
        states.append(m.flags.copy())
        for steps in (1, 4):
            if "uf" in ext:  # UPDATE_FIELDS: rho/u written by every step, compared before update_fields runs
                m.run(1, fx, -1e-5 if fx else 0.0, 2e-5 if fx else 0.0)
                states += [m.rho.copy(), m.u.copy()]
            if mb and steps == 4:  # some walls stop, the others change speed
                solid = (m.flags & 3) == 1
                m.u[:N][solid] *= np.float32(0.5)
                m.u[N:2 * N][solid & (np.arange(N) % 3 == 0)] = 0.0
                m.u[:N][solid & (np.arange(N) % 5 == 0)] = 0.0
                m.u[2 * N:][solid & (np.arange(N) % 5 == 0)] = 0.0
                m.update_moving_boundaries()
                states.append(m.flags.copy())
            m.run(steps, fx, -1e-5 if fx else 0.0, 2e-5 if fx else 0.0)
            m.update_fields(fx, -1e-5 if fx else 0.0, 2e-5 if fx else 0.0)
            states += [m.fi.copy(), m.rho.copy(), m.u.copy()]
            if "ff" in ext:
                m.update_force_field()
                states.append(m.F.copy())
        runs.append(states)
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def test_voxelize_moving_mesh_reconstructs_like_reference():
    """Voxelize with velocity, move the mesh, voxelize again: flags, u and DDFs bit-identical."""
    _harness((19, "srt", "fp32", ()))
    import lbm_cases as LC
    from fluidx3d_gb300.mesh import ellipsoid_mesh
    shape = (40, 34, 30)
    runs = []
    for cls in (oracle.RefHarness, oracle.Oracle):
        m = cls(*shape, q=19, nu=0.05)
        m.initialize()
        for k, shift in enumerate((0.0, 1.7)):
            mesh = ellipsoid_mesh(center=(17.0 + shift, 16.5, 14.2), semi_axes=(9.0, 7.5, 6.0), n_theta=16, n_phi=32, seed=3)
            rot = (0.0, 0.0, 0.01)
            bbu, direction = LC.bbu_for(mesh, center=tuple(mesh.center), lin=(0.01, 0.0, 0.0), rot=rot)
            m.voxelize_mesh(direction, 0x01, mesh.p0.reshape(-1), mesh.p1.reshape(-1), mesh.p2.reshape(-1), bbu, 1 + k)
        runs.append((m.flags.copy(), m.u.copy(), m.fi.copy()))
    for a, b in zip(*runs):
        assert np.array_equal(a, b)
