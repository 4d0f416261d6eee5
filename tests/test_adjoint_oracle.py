"""The FP64 discrete adjoint of the CPU oracle against central finite differences of its FP64
forward run (the FP64 reference for the GPU adjoint; the reference has no adjoint to compare with)."""
import numpy as np
import pytest

import oracle
from fluidx3d_gb300 import setups as S


def channel_problem(collision, Nx=24, Ny=12, Nz=12, seed=3, q=19):
    f = S.sphere_channel(Nx, Ny, Nz, u_in=0.05, radius=2.5, center=(8.0, 6.0, 6.0))
    F = S.box_filter_noise(Nx, Ny, Nz, sigma=1e-4, width=3, seed=seed)
    o = oracle.Oracle(Nx, Ny, Nz, q=q, collision=collision, extensions=("eq", "ff", "vf"), nu=0.02, precision="f64")
    o.rho[:], o.u[:], o.flags[:], o.F[:] = f["rho"], f["u"], f["flags"], F
    o.initialize()
    return o, o.fi.copy()


@pytest.mark.parametrize("collision,kind,q", [("srt", "ke_plane", 19), ("trt", "ke_plane", 19), ("trt", "drag_x", 19), ("trt", "ke_plane", 27)])
def test_fp64_adjoint_matches_central_differences(collision, kind, q):
    o, f0 = channel_problem(collision, q=q)
    steps = 40
    obj = oracle.objective(kind, 28, 40, plane_x=18, marker=0x41)
    force = (2e-6, 0.0, 0.0)
    J, grad = oracle.fp64_adjoint(o, f0, steps, obj, interval=7, force=force)
    assert J == pytest.approx(oracle.fp64_objective(o, f0, steps, obj, force), rel=1e-14)
    rng = np.random.default_rng(11)
    fluid = np.flatnonzero((o.flags & 3) == 0)
    x = fluid % o.Nx
    cells = np.concatenate([rng.choice(fluid, 5, replace=False), rng.choice(fluid[x == 18], 2, replace=False),
                            rng.choice(fluid[x == 17], 1, replace=False)])  # plane cells: F also enters the objective directly
    eps = 1e-6
    for n in cells:
        for d in range(3):
            k = d * o.N + n
            Fp, Fm = o.F.copy(), o.F.copy()
            Fp[k] += eps
            Fm[k] -= eps
            fd = (oracle.fp64_objective(o, f0, steps, obj, force, Fp) - oracle.fp64_objective(o, f0, steps, obj, force, Fm)) / (2 * eps)
            scale = np.max(np.abs(grad))
            assert abs(grad[k] - fd) <= 1e-6 * scale + 1e-9 * abs(fd), (n, d, grad[k], fd)
    assert np.max(np.abs(grad)) > 0


def test_checkpoint_interval_does_not_change_the_gradient():
    o, f0 = channel_problem("trt")
    obj = oracle.objective("ke_plane", 20, 30, plane_x=18)
    J1, g1 = oracle.fp64_adjoint(o, f0, 30, obj, interval=1)
    J2, g2 = oracle.fp64_adjoint(o, f0, 30, obj, interval=30)
    J3, g3 = oracle.fp64_adjoint(o, f0, 30, obj, interval=8)
    assert J1 == J2 == J3
    assert np.array_equal(g1, g2) and np.array_equal(g1, g3)
