"""The oracle's ray-subset voxelization (used to check the large-lattice voxelization on sampled rays)
equals its full voxelization: on all rays exactly, on a subset exactly on those rays' cells."""
import numpy as np

import oracle
import lbm_cases as LC


def test_voxelize_rays_equals_full_voxelization():
    shape, mesh = LC.voxel_mesh_case()
    bbu, d = LC.bbu_for(mesh)
    N = shape[0] * shape[1] * shape[2]
    o = oracle.Oracle(*shape, w=1.0)
    o.voxelize_mesh(d, 0x41, mesh.p0.astype(np.float32), mesh.p1.astype(np.float32), mesh.p2.astype(np.float32), bbu, 0)
    A = [shape[1] * shape[2], shape[2] * shape[0], shape[0] * shape[1]][d]
    full = np.zeros(N, np.uint8)
    oracle.voxelize_rays(shape, full, d, 0x41, mesh.p0, mesh.p1, mesh.p2, bbu, np.arange(A))
    assert np.count_nonzero(full) > 1000 and np.array_equal(full, o.flags)
    rays = np.random.default_rng(0).choice(A, 50, replace=False)
    sub = np.zeros(N, np.uint8)
    oracle.voxelize_rays(shape, sub, d, 0x41, mesh.p0, mesh.p1, mesh.p2, bbu, rays)
    assert d == 0
    rows = sub.reshape(shape[2], shape[1], shape[0])[rays // shape[1], rays % shape[1], :]
    ref = o.flags.reshape(shape[2], shape[1], shape[0])[rays // shape[1], rays % shape[1], :]
    assert np.array_equal(rows, ref) and np.count_nonzero(sub) == np.count_nonzero(rows)
