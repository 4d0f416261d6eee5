"""Validation and measurement runs of the solver on the five reference workloads (the counterpart of
the reference's validation setups, src/setup.cpp:40-187), printing one JSON object per run.

    python -m fluidx3d_gb300.validate tgv          # 64^3 Taylor-Green vortex, SRT FP32, 1000 steps
    python -m fluidx3d_gb300.validate sphere       # 512x256x256 sphere channel, TRT FP16S, drag
    python -m fluidx3d_gb300.validate large        # 2048x1024x1280 FP16C with a voxelized 200k-triangle mesh
    python -m fluidx3d_gb300.validate adjoint      # 128x64x64 channel, dJ/dF of the outlet-plane kinetic energy
    python -m fluidx3d_gb300.validate adjoint_scale  # sphere channel, dJ/dF of the sphere drag, FP16S
    python -m fluidx3d_gb300.validate variants     # sphere channel: time per step of the extension variants

All inputs are synthetic and seeded. Timings use CUDA events on the solver's stream.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np

from . import LBM, TYPE_S, TYPE_E, TYPE_X, setups as S
from .mesh import ellipsoid_mesh


class Timer:
    """CUDA events on the solver's own stream (through the CUDA runtime of the solver library)."""

    def __init__(self, lbm):
        import torch  # noqa: F401 (device events without adding runtime entry points to the C-ABI)
        self.torch = torch
        self.stream = torch.cuda.ExternalStream(lbm.stream())

    def __enter__(self):
        self.a = self.torch.cuda.Event(enable_timing=True)
        self.b = self.torch.cuda.Event(enable_timing=True)
        self.a.record(self.stream)
        return self

    def __exit__(self, *exc):
        self.b.record(self.stream)
        self.b.synchronize()
        self.ms = self.a.elapsed_time(self.b)


def kinetic_energy(lbm):
    lbm.rho.read_from_device()
    lbm.u.read_from_device()
    N = lbm.get_N()
    u = lbm.u.data.astype(np.float64)
    return 0.5 * float(np.sum(lbm.rho.data.astype(np.float64) * (u[:N] ** 2 + u[N:2 * N] ** 2 + u[2 * N:] ** 2)))


def tgv(N=64, steps=1000, every=100, storage="fp32", collision="srt", arithmetic="auto"):
    """3D Taylor-Green vortex: kinetic-energy decay rate against the low-Re analytic 6 nu k^2."""
    nu = 1.0 / 30.0
    f = S.taylor_green(N, N, N)
    with LBM(N, N, N, nu, collision=collision, storage=storage, arithmetic=arithmetic) as lbm:  # timed run, no readback
        lbm.rho.data[:], lbm.u.data[:] = f["rho"], f["u"]
        lbm.run(0)
        with Timer(lbm) as t:
            lbm.run(steps)
    E = []
    with LBM(N, N, N, nu, collision=collision, storage=storage, arithmetic=arithmetic) as lbm:  # energies along the run
        lbm.rho.data[:], lbm.u.data[:] = f["rho"], f["u"]
        lbm.run(0)
        E.append(kinetic_energy(lbm))
        for _ in range(steps // every):
            lbm.run(every)
            E.append(kinetic_energy(lbm))
    k = 2.0 * math.pi / N
    t_axis = np.arange(len(E)) * every
    rate = -np.polyfit(t_axis[1:], np.log(np.asarray(E[1:])), 1)[0]
    return dict(run="tgv", N=N, steps=steps, storage=storage, energies=E, decay_rate=float(rate), analytic_rate=6.0 * float(np.float32(nu)) * k * k,
                mlups=N ** 3 * steps / (t.ms * 1e-3) / 1e6)


def sphere_setup(storage="fp16s", collision="trt", extensions=("eq",), arithmetic="auto", Nx=512, Ny=256, Nz=256, radius=32.0,
                 center=(128.0, 128.0, 128.0), u_in=0.075, Re=100.0, F=None, fx=0.0):
    nu = u_in * 2.0 * radius / Re
    f = S.sphere_channel(Nx, Ny, Nz, u_in=u_in, radius=radius, center=center)
    lbm = LBM(Nx, Ny, Nz, nu, fx, 0.0, 0.0, collision=collision, storage=storage, extensions=extensions, arithmetic=arithmetic)
    lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:] = f["rho"], f["u"], f["flags"]
    if F is not None:
        lbm.F.data[:] = F
    return lbm


def sphere(storage="fp16s", steps=20000, every=1000, collision="trt", arithmetic="auto"):
    """512x256x256 channel, sphere r=32, Re=100: drag (FP64 reduction) along the run, MLUPs/s."""
    with sphere_setup(storage, collision, arithmetic=arithmetic) as lbm:
        lbm.run(0)
        drag, ms = [], 0.0
        for _ in range(steps // every):
            with Timer(lbm) as t:
                lbm.run(every)
            ms += t.ms
            drag.append(lbm.object_force(TYPE_S | TYPE_X).tolist())
        lbm.u.read_from_device()
        N = lbm.get_N()
        u = lbm.u.data.copy()
        fluid = int(np.count_nonzero((lbm.flags.data & 3) != 1))
        return dict(run="sphere", storage=storage, collision=collision, steps=steps, drag=drag, mlups=N * steps / (ms * 1e-3) / 1e6,
                    fluid_mlups=fluid * steps / (ms * 1e-3) / 1e6, ux_mean=float(np.mean(u[:N][(lbm.flags.data & 3) == 0]))), u


def large(steps=2000, triangles=200_000, arithmetic="auto"):
    """2048x1024x1280 FP16C (147.6 GB on the device): seeded procedural ellipsoid mesh voxelized on the
    device, TYPE_E inlet/outlet at u=0.05, nu=1e-4, SRT; MLUPs/s over `steps`."""
    Nx, Ny, Nz = 2048, 1024, 1280
    n_theta = int(round(math.sqrt(triangles / 2.0 / 1.6)))
    n_phi = int(round(triangles / 2.0 / n_theta))
    mesh = ellipsoid_mesh(center=(600.0, Ny / 2.0, Nz / 2.0), semi_axes=(300.0, 120.0, 120.0), n_theta=n_theta, n_phi=n_phi,
                          noise_amplitude=8.0, smooth_width=9, seed=2024)
    lbm = LBM(Nx, Ny, Nz, 1e-4, storage="fp16c", extensions=("eq",), arithmetic=arithmetic)
    try:
        t0 = time.perf_counter()
        lbm.voxelize_mesh_on_device(mesh, TYPE_S | TYPE_X)
        lbm.synchronize()
        t_vox = time.perf_counter() - t0
        flags = lbm.flags.data
        fl3 = flags.reshape(Nz, Ny, Nx)
        for xs in (0, Nx - 1):  # TYPE_E inlet and outlet planes
            plane = fl3[:, :, xs]
            plane[plane == 0] = TYPE_E
        lbm.u.x[:] = np.float32(0.05)
        lbm.u.x[(flags & TYPE_S) != 0] = 0.0
        lbm.run(0)
        lbm.run(10)
        with Timer(lbm) as t:
            lbm.run(steps)
        solid = int(np.count_nonzero((flags & 3) == 1))
        return dict(run="large", cells=lbm.get_N(), triangles=mesh.triangle_number, solid_cells=solid, voxelize_s=t_vox, steps=steps,
                    mlups=lbm.get_N() * steps / (t.ms * 1e-3) / 1e6, fluid_mlups=(lbm.get_N() - solid) * steps / (t.ms * 1e-3) / 1e6,
                    device_bytes_per_cell=lbm.bytes_per_cell_device()), (lbm, mesh)
    except Exception:
        lbm.close()
        raise


def adjoint_setup(storage="fp32", Nx=128, Ny=64, Nz=64, sigma=1e-5, seed=4, collision="srt"):
    """Channel with TYPE_E inlet/outlet at u=0.05 and TYPE_S walls, tau=0.56; F = seeded Gaussian noise
    (sigma) smoothed by a 5-cell box filter."""
    nu = (0.56 - 0.5) / 3.0
    f = S.sphere_channel(Nx, Ny, Nz, u_in=0.05)
    F = S.box_filter_noise(Nx, Ny, Nz, sigma=sigma, width=5, seed=seed)
    lbm = LBM(Nx, Ny, Nz, nu, 0.0, 0.0, 0.0, collision=collision, storage=storage, extensions=("eq", "ff", "vf"))
    lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:], lbm.F.data[:] = f["rho"], f["u"], f["flags"], F
    return lbm


def adjoint(steps=2000, window=None, plane_x=120, interval=100):
    """dJ/dF, J = mean kinetic energy on plane x=120 over steps 1800-2000 (the last tenth of the run);
    adjoint/forward time ratio."""
    window = window or (steps - steps // 10, steps)
    with adjoint_setup() as lbm:
        J, grad, st = lbm.run_adjoint(steps, "ke_plane", window=window, plane_x=plane_x, checkpoint_interval=interval)
    with adjoint_setup() as lbm:
        lbm.run(0)
        with Timer(lbm) as t:
            lbm.run(steps)
    total = st["forward_ms"] + st["reverse_ms"]
    return dict(run="adjoint", J=J, grad_norm=float(np.linalg.norm(grad)), stats=st, forward_only_ms=t.ms,
                gradient_over_forward=total / t.ms), grad


def adjoint_scale(steps=10000, window=None, interval=200, storage="fp16s"):
    """dJ/dF on the sphere channel, J = x drag on the sphere averaged over steps 9000-10000 (the last
    tenth of the run), F = 0."""
    window = window or (steps - steps // 10, steps)
    with sphere_setup(storage, "trt", extensions=("eq", "ff", "vf")) as lbm:
        J, grad, st = lbm.run_adjoint(steps, "drag_x", window=window, marker=TYPE_S | TYPE_X, checkpoint_interval=interval)
    with sphere_setup(storage, "trt", extensions=("eq", "ff", "vf")) as lbm:
        lbm.run(0)
        with Timer(lbm) as t:
            lbm.run(steps)
    total = st["forward_ms"] + st["reverse_ms"]
    return dict(run="adjoint_scale", storage=storage, J=J, grad_norm=float(np.linalg.norm(grad)), stats=st, forward_only_ms=t.ms,
                gradient_over_forward=total / t.ms), grad


VARIANTS = [("fp16s", ("eq",)), ("fp16s", ("eq", "mb")), ("fp16s", ("eq", "sg")), ("fp16s", ("eq", "mb", "sg")),
            ("fp16c", ("eq", "mb")), ("fp32", ("eq",)), ("fp32", ("eq", "mb"))]


def variants(steps=200, warmup=20, sphere_uy=0.02):
    """The C2 sphere channel (512x256x256, D3Q19 TRT, automatic arithmetic and kernel) with the
    SUBGRID / MOVING_BOUNDARIES variants; with MOVING_BOUNDARIES the sphere moves at u_y = sphere_uy.
    Per variant: ms per step over `steps` steps after `warmup`, MLUPs/s, the TYPE_MS cell count and
    the fraction of the measured HBM peak under the reference's byte accounting."""
    import os
    peak = None
    try:
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        with open(os.path.join(root, "MEASURED_PEAKS.json")) as fh:
            peak = float(json.load(fh)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        pass
    Nx, Ny, Nz = 512, 256, 256
    N = Nx * Ny * Nz
    f = S.sphere_channel(Nx, Ny, Nz, u_in=0.075, radius=32.0, center=(128.0, 128.0, 128.0))
    moving_u = f["u"].copy()
    moving_u[N:2 * N][(f["flags"] & TYPE_X) != 0] = np.float32(sphere_uy)
    out = []
    for storage, ext in VARIANTS:
        with LBM(Nx, Ny, Nz, 0.048, collision="trt", storage=storage, extensions=ext) as lbm:
            lbm.rho.data[:], lbm.flags.data[:] = f["rho"], f["flags"]
            lbm.u.data[:] = moving_u if "mb" in ext else f["u"]
            lbm.run(warmup)
            with Timer(lbm) as t:
                lbm.run(steps)
            ms = t.ms / steps
            marked = 0
            if "mb" in ext:
                lbm.flags.read_from_device()
                marked = int(np.count_nonzero((lbm.flags.data & 3) == 3))
            bpc = lbm.bandwidth_bytes_per_cell()
            r = dict(storage=storage, extensions=list(ext), ms_per_step=ms, mlups=N / (ms * 1e-3) / 1e6, ms_cells=marked,
                     bytes_per_cell=bpc)
            if peak:
                r["hbm_fraction"] = bpc * N / (ms * 1e-3) / 1e9 / peak
            out.append(r)
    return dict(run="variants", cells=N, steps=steps, results=out)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("run", choices=["tgv", "sphere", "large", "adjoint", "adjoint_scale", "variants"])
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--storage", default=None)
    args = ap.parse_args(argv)
    kw = {}
    if args.steps is not None:
        kw["steps"] = args.steps
    if args.storage is not None:
        kw["storage"] = args.storage
    if args.run == "tgv":
        out = tgv(**kw)
    elif args.run == "sphere":
        out = sphere(**kw)[0]
    elif args.run == "large":
        out, (lbm, _) = large(**{k: v for k, v in kw.items() if k != "storage"})
        lbm.close()
    elif args.run == "adjoint":
        out = adjoint(**{k: v for k, v in kw.items() if k != "storage"})[0]
    elif args.run == "variants":
        out = variants(**{k: v for k, v in kw.items() if k != "storage"})
    else:
        out = adjoint_scale(**kw)[0]
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
