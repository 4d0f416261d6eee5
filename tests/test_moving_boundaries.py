"""MOVING_BOUNDARIES in the CPU oracle: the analytic plane Couette profile between a wall at rest
and a moving wall, and the TYPE_MS marking rules of initialize and update_moving_boundaries
(src/kernel.cpp:1104-1113, 1378-1387, 1431-1450). The oracle's bit-parity with the reference's own
kernels is pinned in test_oracle_vs_reference.py and test_oracle_golden.py."""
import numpy as np
import pytest

import oracle


def plane_couette(Nx=4, Ny=4, Nz=18, U=0.05):
    """Periodic in x and y; TYPE_S planes z=0 (at rest) and z=Nz-1 (u_x = U)."""
    N = Nx * Ny * Nz
    z = np.arange(N) // (Nx * Ny)
    flags = np.zeros(N, np.uint8)
    flags[(z == 0) | (z == Nz - 1)] = 0x01
    u = np.zeros(3 * N, np.float32)
    u[:N][z == Nz - 1] = U
    return (Nx, Ny, Nz), flags, u


@pytest.mark.parametrize("precision,tol", [("f64", 1e-6), ("f32", 5e-5)])
def test_plane_couette_profile(precision, tol):
    """Steady state u_x(z) = U (z - 1/2) / (Nz - 2): the walls sit halfway between the solid and the
    first fluid cell (bounce-back), the moving wall's momentum enters through the TYPE_MS cells."""
    shape, flags, u = plane_couette()
    Nx, Ny, Nz = shape
    N = Nx * Ny * Nz
    o = oracle.Oracle(*shape, q=19, collision="srt", extensions=("mb",), nu=1.0 / 6.0, precision=precision)
    o.u[:], o.flags[:] = u, flags
    o.initialize()
    z = np.arange(N) // (Nx * Ny)
    assert np.all(((o.flags & 3) == 3) == (z == Nz - 2))  # only the cells below the moving wall are marked
    o.run(8000)
    o.update_fields()
    ux = o.u[:N].reshape(Nz, Ny, Nx)
    exact = 0.05 * (np.arange(Nz) - 0.5) / (Nz - 2)
    err = np.max(np.abs(ux[1:-1] - exact[1:-1, None, None])) / 0.05
    assert err < tol, err


def test_without_moving_boundaries_the_wall_velocity_is_ignored():
    """Without the extension, solid cells are reset to rest and no momentum enters."""
    shape, flags, u = plane_couette()
    o = oracle.Oracle(*shape, q=19, collision="srt", nu=1.0 / 6.0)
    o.u[:], o.flags[:] = u, flags
    o.initialize()
    o.run(200)
    o.update_fields()
    assert np.max(np.abs(o.u)) == 0.0
    assert np.count_nonzero((o.flags & 3) == 3) == 0


@pytest.mark.parametrize("q", [19, 27])
def test_marking_rules(q):
    """initialize marks TYPE_T cells too, update_moving_boundaries leaves TYPE_T cells as they are;
    TYPE_E cells are never marked; a solid with u = 0 marks nothing; a solid whose neighbours are all
    solid comes to rest at initialize."""
    Nx, Ny, Nz = 9, 8, 7
    N = Nx * Ny * Nz
    rng = np.random.default_rng(5)
    flags = rng.choice(np.array([0, 0, 0, 0x01, 0x01, 0x02, 0x03, 0x04, 0x41], np.uint8), N)
    u = rng.normal(0, 0.02, 3 * N).astype(np.float32)
    still = rng.random(N) < 0.3
    for d in range(3):
        u[d * N:(d + 1) * N][still] = 0.0
    o = oracle.Oracle(Nx, Ny, Nz, q=q, extensions=("mb",), nu=0.05)
    o.u[:], o.flags[:] = u, flags
    o.initialize()
    after_init = o.flags.copy()
    o.update_moving_boundaries()
    changed = after_init != o.flags
    assert np.all((flags[changed] & 0x04) != 0)  # only TYPE_T cells differ between the two rules
    assert np.all((o.flags[(flags & 3) == 2] & 3) == 2)  # TYPE_E stays TYPE_E
    assert np.all((o.flags[(flags & 3) == 1] & 3) == 1)  # solids stay solid
    # brute-force rule on the update's result
    x, y, z = np.arange(N) % Nx, (np.arange(N) // Nx) % Ny, np.arange(N) // (Nx * Ny)
    moving = ((flags & 3) == 1) & ((o.u[:N] != 0) | (o.u[N:2 * N] != 0) | (o.u[2 * N:] != 0))
    dirs = [(a, b, cc) for a in (-1, 0, 1) for b in (-1, 0, 1) for cc in (-1, 0, 1) if (a, b, cc) != (0, 0, 0)]
    if q == 19:
        dirs = [d for d in dirs if sum(abs(v) for v in d) <= 2]
    near = np.zeros(N, bool)
    for a, b, cc in dirs:
        j = (x + a) % Nx + ((y + b) % Ny + ((z + cc) % Nz) * Ny) * Nx
        near |= moving[j]
    target = ((flags & 3) != 1) & ((flags & 3) != 2) & ((flags & 0x04) == 0)
    expect = np.where(near, flags | 3, flags & ~np.uint8(3)).astype(np.uint8)
    assert np.array_equal(o.flags[target], expect[target])
