"""Accuracy of the GPU solver against the FP64 oracle on the reference workloads, and of FP16S against
FP32 DDF storage at full size; prints one JSON object. A test-side tool (it uses the oracle), run
on a GPU machine:

    python tests/report_accuracy.py            # C1 TGV and the C2 geometry at quarter scale
    python tests/report_accuracy.py --full-c2  # also C2 at full size, FP16S against FP32 storage
    python tests/report_accuracy.py --only-c3-voxel  # C3 voxel flags on sampled rays against the oracle

Errors are max-norms relative to max|u| of the reference field and L2 norms relative to the
reference's L2 norm (u over fluid cells), and the relative difference of the FP64-summed sphere drag.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from fluidx3d_gb300 import LBM, TYPE_S, TYPE_X, setups as S  # noqa: E402

MARKER = TYPE_S | TYPE_X


def rel_u(u, ref, mask=None):
    """max-norm of u - ref relative to max|ref|"""
    u = u.astype(np.float64).reshape(3, -1)
    ref = ref.astype(np.float64).reshape(3, -1)
    if mask is not None:
        u, ref = u[:, mask], ref[:, mask]
    return float(np.max(np.abs(u - ref)) / np.max(np.abs(ref)))


def rms_u(u, ref, mask=None):
    """L2 norm of u - ref relative to the L2 norm of ref"""
    u = u.astype(np.float64).reshape(3, -1)
    ref = ref.astype(np.float64).reshape(3, -1)
    if mask is not None:
        u, ref = u[:, mask], ref[:, mask]
    return float(np.sqrt(np.sum((u - ref) ** 2) / np.sum(ref ** 2)))


def gpu_run(shape, nu, fields, steps, storage, arithmetic, collision="srt", extensions=(), drag=False):
    with LBM(*shape, nu, collision=collision, storage=storage, extensions=extensions, arithmetic=arithmetic) as lbm:
        lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:] = fields["rho"], fields["u"], fields["flags"]
        lbm.run(steps)
        lbm.u.read_from_device()
        out = dict(u=lbm.u.data.copy())
        if drag:
            out["drag"] = np.asarray(lbm.object_force(MARKER), dtype=np.float64)
        return out


def oracle_run(shape, nu, fields, steps, collision="srt", extensions=(), drag=False):
    o = oracle.Oracle(*shape, q=19, collision=collision, extensions=extensions, nu=nu, precision="f64")
    o.rho[:], o.u[:], o.flags[:] = fields["rho"], fields["u"], fields["flags"]
    o.initialize()
    o.run(steps)
    o.update_fields()
    out = dict(u=o.u.copy())
    if drag:
        o.update_force_field()
        out["drag"] = o.object_sum(1, MARKER)[:3]
    return out


def c1_tgv(steps=1000):
    shape, nu = (64, 64, 64), 1.0 / 30.0
    f = S.taylor_green(*shape)
    ref = oracle_run(shape, nu, f, steps)
    res = {}
    for storage, arith in (("fp32", "exact"), ("fp32", "fast"), ("fp16s", "exact"), ("fp16s", "fast"), ("fp16c", "exact"), ("fp16c", "fast")):
        g = gpu_run(shape, nu, f, steps, storage, arith)
        res[f"{storage}_{arith}"] = dict(max=rel_u(g["u"], ref["u"]), rms=rms_u(g["u"], ref["u"]))
    return dict(workload="64^3 Taylor-Green, D3Q19 SRT, 1000 steps", u_err_vs_fp64=res)


def c2_quarter(steps=2000):
    shape = (128, 64, 64)
    nu = 0.075 * 16.0 / 100.0  # Re = 100 on the sphere diameter 16
    f = S.sphere_channel(*shape, u_in=0.075, radius=8.0, center=(32.0, 32.0, 32.0))
    fluid = (f["flags"] & 3) == 0
    kw = dict(collision="trt", extensions=("eq",), drag=True)
    ref = oracle_run(shape, nu, f, steps, **kw)
    res = {}
    for storage, arith in (("fp32", "exact"), ("fp32", "fast"), ("fp16s", "exact"), ("fp16s", "fast"), ("fp16c", "exact"), ("fp16c", "fast")):
        g = gpu_run(shape, nu, f, steps, storage, arith, **kw)
        res[f"{storage}_{arith}"] = dict(u_err_vs_fp64=rel_u(g["u"], ref["u"], fluid), u_rms_err_vs_fp64=rms_u(g["u"], ref["u"], fluid),
                                          drag_rel_err_vs_fp64=float(abs(g["drag"][0] - ref["drag"][0]) / abs(ref["drag"][0])),
                                          drag_x=float(g["drag"][0]))
    return dict(workload="128x64x64 sphere channel (C2 geometry at quarter scale, r=8), D3Q19 TRT EQ, 2000 steps",
                fp64_drag_x=float(ref["drag"][0]), results=res)


def c2_full(steps=20000):
    shape, nu = (512, 256, 256), 0.048
    f = S.sphere_channel(*shape, u_in=0.075, radius=32.0, center=(128.0, 128.0, 128.0))
    fluid = (f["flags"] & 3) == 0
    kw = dict(collision="trt", extensions=("eq",), drag=True)
    a = gpu_run(shape, nu, f, steps, "fp32", "exact", **kw)
    b = gpu_run(shape, nu, f, steps, "fp16s", "auto", **kw)
    return dict(workload="512x256x256 sphere channel (C2), D3Q19 TRT EQ, 20000 steps",
                fp16s_u_err_vs_fp32=rel_u(b["u"], a["u"], fluid), fp16s_u_rms_err_vs_fp32=rms_u(b["u"], a["u"], fluid),
                fp16s_drag_rel_diff_vs_fp32=float(abs(b["drag"][0] - a["drag"][0]) / abs(a["drag"][0])),
                drag_x_fp32=float(a["drag"][0]), drag_x_fp16s=float(b["drag"][0]))


def c3_voxel(samples=4096, seed=11):
    """C3 voxelization (2048x1024x1280, seeded 200k-triangle ellipsoid as in the large validation run)
    on the GPU against the FP32 voxelizer restatement on `samples` random rays through the mesh box:
    the flags of every cell of those rays must be identical."""
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import math
    import lbm_cases as LC
    from fluidx3d_gb300.mesh import ellipsoid_mesh
    Nx, Ny, Nz = 2048, 1024, 1280
    triangles = 200_000
    n_theta = int(round(math.sqrt(triangles / 2.0 / 1.6)))
    n_phi = int(round(triangles / 2.0 / n_theta))
    mesh = ellipsoid_mesh(center=(600.0, Ny / 2.0, Nz / 2.0), semi_axes=(300.0, 120.0, 120.0), n_theta=n_theta, n_phi=n_phi,
                          noise_amplitude=8.0, smooth_width=9, seed=2024)
    bbu, direction = LC.bbu_for(mesh)
    assert direction == 0
    with LBM(Nx, Ny, Nz, 1e-4, storage="fp16c", extensions=("eq",)) as lbm:
        lbm.voxelize_mesh_on_device(mesh, MARKER)  # not initialized: flags are read back
        g = lbm.flags.data.reshape(Nz, Ny, Nx)
        rng = np.random.default_rng(seed)
        y = rng.integers(max(0, int(bbu[2])), min(Ny, int(bbu[5]) + 1), samples)
        z = rng.integers(max(0, int(bbu[3])), min(Nz, int(bbu[6]) + 1), samples)
        rows_gpu = g[z, y, :].copy()
    flags = np.zeros(Nx * Ny * Nz, np.uint8)
    oracle.voxelize_rays((Nx, Ny, Nz), flags, 0, MARKER, mesh.p0, mesh.p1, mesh.p2, bbu, y.astype(np.uint64) + z.astype(np.uint64) * Ny)
    rows_cpu = flags.reshape(Nz, Ny, Nx)[z, y, :]
    return dict(workload="C3 voxelization, 2048x1024x1280, 200k-triangle seeded ellipsoid", rays=samples, cells_compared=int(rows_cpu.size),
                solid_cells_in_rays=int(np.count_nonzero(rows_cpu)), mismatches=int(np.count_nonzero(rows_gpu != rows_cpu)),
                triangles=int(mesh.triangle_number))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--full-c2", action="store_true")
    ap.add_argument("--c3-voxel", action="store_true", help="C3 voxelization on sampled rays (148 GB on the GPU, 45 GB host)")
    ap.add_argument("--only-c3-voxel", action="store_true")
    args = ap.parse_args(argv)
    out = {}
    if not args.only_c3_voxel:
        out.update(c1=c1_tgv(), c2_quarter=c2_quarter())
        if args.full_c2:
            out["c2_full"] = c2_full()
    if args.c3_voxel or args.only_c3_voxel:
        out["c3_voxel"] = c3_voxel()
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
