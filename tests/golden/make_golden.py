"""Generates the golden fixtures in tests/golden/ from the reference's own kernels.

The generator runs the reference's OpenCL C kernel text compiled for the CPU (oracle/ref_harness,
built from the reference sources by oracle/ref_harness/build_ref.py) on every case of
tests/lbm_cases.py and stores what it produced. It needs the reference tree and is run by hand:

    python tests/golden/make_golden.py              # every fixture
    python tests/golden/make_golden.py CASE [CASE]  # only the lbm_<case>.npz fixtures named

Fixtures:
  lbm_<case>.npz   rho, u (after update_fields), F (after update_force_field, FORCE_FIELD cases),
                   flags (MOVING_BOUNDARIES cases: TYPE_MS marked by initialize) and sha256 of the raw
                   DDF bytes, after case.steps time steps
  tgv64.npz        Taylor-Green 64^3 D3Q19 SRT FP32 tau=0.6 after 1000 steps: sha256 of rho/u
                   bytes, u_x at the box centre (the reference's own "binary identity" probe,
                   src/setup.cpp:58), kinetic energy, and a strided sample of u
  voxel.npz        flags after voxelizing the seeded bumpy ellipsoid of lbm_cases.voxel_mesh_case
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle.ref_harness import build_ref  # noqa: E402
import lbm_cases as LC  # noqa: E402


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(case, threads=None):
    h = oracle.RefHarness(*case.shape, q=case.q, collision=case.collision, storage=case.storage, extensions=case.extensions,
                          nu=case.nu, threads=threads)
    f = case.fields()
    h.rho[:], h.u[:], h.flags[:], h.F[:] = f["rho"], f["u"], f["flags"], f["F"]
    h.initialize()
    h.run(case.steps, *case.force)
    case.settle_fields(h)
    if "ff" in case.extensions:
        h.update_force_field()
    return h


def main(names=None):
    build_ref.build_all()
    for case in LC.CASES:
        if names and case.name not in names:
            continue
        h = run_case(case)
        out = dict(rho=h.rho, u=h.u, fi_sha256=np.array(sha(h.fi)), steps=np.array(case.steps))
        if "ff" in case.extensions:
            out["F"] = h.F
        if "mb" in case.extensions:
            out["flags"] = h.flags
        np.savez_compressed(os.path.join(HERE, f"lbm_{case.name}.npz"), **out)
        print("wrote", case.name)
    if names:
        return
    c = LC.TGV64
    h = run_case(c)
    Nx, Ny, Nz = c.shape
    n_center = Nx // 2 + (Ny // 2 + (Nz // 2) * Ny) * Nx
    ux, uy, uz = h.u[:h.N], h.u[h.N:2 * h.N], h.u[2 * h.N:]
    ke = 0.5 * np.sum(h.rho.astype(np.float64) * (ux.astype(np.float64) ** 2 + uy.astype(np.float64) ** 2 + uz.astype(np.float64) ** 2))
    np.savez_compressed(os.path.join(HERE, "tgv64.npz"), rho_sha256=np.array(sha(h.rho)), u_sha256=np.array(sha(h.u)),
                        ux_center=np.float32(ux[n_center]), kinetic_energy=np.float64(ke), u_sample=h.u[::97].copy(),
                        rho_sample=h.rho[::97].copy(), fi_sha256=np.array(sha(h.fi)))
    print("wrote tgv64 ux_center", ux[n_center])
    shape, mesh = LC.voxel_mesh_case()
    for storage in ("fp32",):
        h = oracle.RefHarness(*shape, q=19, collision="srt", storage=storage, nu=0.1)
        bbu, direction = LC.bbu_for(mesh)
        h.voxelize_mesh(direction, 0x01, mesh.p0.reshape(-1), mesh.p1.reshape(-1), mesh.p2.reshape(-1), bbu, 1)
        np.savez_compressed(os.path.join(HERE, "voxel.npz"), flags=h.flags, direction=np.array(direction), bbu=bbu,
                            solid_cells=np.array(int(np.sum(h.flags == 1))))
        print("wrote voxel", direction, int(np.sum(h.flags == 1)))


if __name__ == "__main__":
    main(sys.argv[1:])
