"""Synthetic initial conditions for the workloads the solver is measured and checked on.

Each builder returns host arrays in the reference's layout (rho N, u 3N SoA, flags N uint8, F 3N
SoA, float32) for a grid ``Nx x Ny x Nz`` with n = x+(y+z*Ny)*Nx. They mirror the reference's own
setups (src/setup.cpp) where one exists:
  * ``taylor_green``: 3D Taylor-Green vortex (src/setup.cpp:40-59 pattern) with the analytic
    low-Re density field, cell-centre coordinates x+0.5;
  * ``sphere_channel``: x-channel with TYPE_E inlet/outlet planes, TYPE_S y/z walls and a TYPE_S
    sphere (src/shapes.cpp:5-8 ``sphere``) marked TYPE_S|TYPE_X for force summation
    (src/setup.cpp:148-187 pattern);
  * ``empty_box``: the reference benchmark's periodic empty box (src/setup.cpp:5-36);
  * ``lid_driven_cavity`` and ``taylor_couette``: the reference's MOVING_BOUNDARIES setups
    (src/setup.cpp:236-247 and 212-229), solid walls with a velocity.
"""
from __future__ import annotations

import numpy as np

TYPE_S, TYPE_E, TYPE_T, TYPE_F, TYPE_I, TYPE_G, TYPE_X, TYPE_Y = 0x01, 0x02, 0x04, 0x08, 0x10, 0x20, 0x40, 0x80


def coords(Nx, Ny, Nz):
    z, y, x = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    return x.reshape(-1), y.reshape(-1), z.reshape(-1)


def empty_box(Nx, Ny, Nz):
    N = Nx * Ny * Nz
    return dict(rho=np.ones(N, np.float32), u=np.zeros(3 * N, np.float32), flags=np.zeros(N, np.uint8),
                F=np.zeros(3 * N, np.float32))


def taylor_green(Nx, Ny, Nz, u0=0.05, rho0=1.0):
    """u_x = u0 sin(kx)cos(ky)cos(kz), u_y = -u0 cos(kx)sin(ky)cos(kz), u_z = 0,
    rho = rho0 + 3 rho0 u0^2/16 (cos 2kx + cos 2ky)(cos 2kz + 2), k = 2 pi / N per axis."""
    x, y, z = coords(Nx, Ny, Nz)
    kx, ky, kz = 2 * np.pi / Nx * (x + 0.5), 2 * np.pi / Ny * (y + 0.5), 2 * np.pi / Nz * (z + 0.5)
    ux = u0 * np.sin(kx) * np.cos(ky) * np.cos(kz)
    uy = -u0 * np.cos(kx) * np.sin(ky) * np.cos(kz)
    uz = np.zeros_like(ux)
    rho = rho0 + 3.0 * rho0 * u0 ** 2 / 16.0 * (np.cos(2 * kx) + np.cos(2 * ky)) * (np.cos(2 * kz) + 2.0)
    N = Nx * Ny * Nz
    return dict(rho=rho.astype(np.float32), u=np.concatenate([ux, uy, uz]).astype(np.float32),
                flags=np.zeros(N, np.uint8), F=np.zeros(3 * N, np.float32))


def sphere_mask(Nx, Ny, Nz, center, radius):
    """src/shapes.cpp:5-8: (x,y,z)-p squared distance <= r^2, evaluated in FP32."""
    x, y, z = coords(Nx, Ny, Nz)
    c = np.asarray(center, np.float32)
    tx = x.astype(np.float32) - c[0]
    ty = y.astype(np.float32) - c[1]
    tz = z.astype(np.float32) - c[2]
    return (tx * tx + ty * ty) + tz * tz <= np.float32(radius) * np.float32(radius)


def sphere_channel(Nx, Ny, Nz, u_in=0.075, radius=None, center=None, walls=True, sphere_flags=TYPE_S | TYPE_X):
    """x-channel: TYPE_E planes x=0 and x=Nx-1 at (u_in,0,0), rho=1; TYPE_S walls y,z in {0,N-1};
    TYPE_S|TYPE_X sphere. Fluid starts at rest except on the TYPE_E planes... and everywhere at
    u_in so the run starts from a uniform stream."""
    N = Nx * Ny * Nz
    x, y, z = coords(Nx, Ny, Nz)
    flags = np.zeros(N, np.uint8)
    if walls:
        flags[(y == 0) | (y == Ny - 1) | (z == 0) | (z == Nz - 1)] = TYPE_S
    eq = ((x == 0) | (x == Nx - 1)) & (flags == 0)
    flags[eq] = TYPE_E
    if radius is not None:
        if center is None:
            center = (Nx / 4.0, Ny / 2.0, Nz / 2.0)
        flags[sphere_mask(Nx, Ny, Nz, center, radius)] = sphere_flags
    u = np.zeros(3 * N, np.float32)
    fluid_or_e = (flags & TYPE_S) == 0
    u[:N][fluid_or_e] = u_in
    return dict(rho=np.ones(N, np.float32), u=u, flags=flags, F=np.zeros(3 * N, np.float32))


def box_filter_noise(Nx, Ny, Nz, sigma, width=5, seed=0):
    """Seeded Gaussian noise (3 components) smoothed by a periodic box filter of the given width."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(3):
        a = rng.normal(0.0, sigma, size=(Nz, Ny, Nx))
        for axis in range(3):
            acc = np.zeros_like(a)
            for s in range(-(width // 2), width // 2 + 1):
                acc += np.roll(a, s, axis=axis)
            a = acc / width
        out.append(a.reshape(-1))
    return np.concatenate(out).astype(np.float32)


def lid_driven_cavity(Nx, Ny, Nz, u_lid=0.1):
    """src/setup.cpp:236-247: TYPE_S on all six faces, u_y = u_lid on the plane z = Nz-1 (the moving
    lid; with MOVING_BOUNDARIES the cells below it become TYPE_MS)."""
    N = Nx * Ny * Nz
    x, y, z = coords(Nx, Ny, Nz)
    flags = np.zeros(N, np.uint8)
    flags[(x == 0) | (x == Nx - 1) | (y == 0) | (y == Ny - 1) | (z == 0) | (z == Nz - 1)] = TYPE_S
    u = np.zeros(3 * N, np.float32)
    u[N:2 * N][z == Nz - 1] = np.float32(u_lid)
    return dict(rho=np.ones(N, np.float32), u=u, flags=flags, F=np.zeros(3 * N, np.float32))


def _z_cylinder(Nx, Ny, Nz, radius):
    """src/shapes.cpp:21-26 cylinder() about the box centre with axis (0,0,Nz), in FP32 and the
    reference's operation order: (tx^2+ty^2+tz^2) - tz^2 <= r^2."""
    x, y, z = coords(Nx, Ny, Nz)
    f = np.float32
    tx = x.astype(f) - f(0.5 * Nx - 0.5)
    ty = y.astype(f) - f(0.5 * Ny - 0.5)
    tz = z.astype(f) - f(0.5 * Nz - 0.5)
    sqnt = tz * tz
    dist = ((tx * tx + ty * ty) + tz * tz) - sqnt
    r = f(radius)
    return (dist <= r * r) & (sqnt <= f(0.5 * Nz) * f(0.5 * Nz))


def taylor_couette(Nx, Ny, Nz, seed=42):
    """src/setup.cpp:212-229: TYPE_S outside the cylinder of radius Nx/2-1 (at rest) and inside the
    cylinder of radius Nx/4, which rotates: u = (p_y, -p_x, small noise) with p the box-relative
    position in [-0.5, 0.5]^3 (src/lbm.hpp:528-530). The noise on u_z (+-0.001) is seeded numpy noise in
    place of the reference's own generator."""
    N = Nx * Ny * Nz
    x, y, z = coords(Nx, Ny, Nz)
    flags = np.zeros(N, np.uint8)
    flags[~_z_cylinder(Nx, Ny, Nz, Nx // 2 - 1)] = TYPE_S
    inner = _z_cylinder(Nx, Ny, Nz, Nx // 4)
    f = np.float32
    px = (x.astype(f) + f(0.5)) / f(Nx) - f(0.5)
    py = (y.astype(f) + f(0.5)) / f(Ny) - f(0.5)
    rng = np.random.default_rng(seed)
    u = np.zeros(3 * N, np.float32)
    u[:N][inner] = py[inner]
    u[N:2 * N][inner] = -px[inner]
    u[2 * N:][inner] = ((1.0 - rng.uniform(0.0, 2.0, N)) * 0.001).astype(np.float32)[inner]
    flags[inner] = TYPE_S
    return dict(rho=np.ones(N, np.float32), u=u, flags=flags, F=np.zeros(3 * N, np.float32))
