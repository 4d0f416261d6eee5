"""Mesh voxelization on the GPU: flags bit-identical to the reference's fixture and to the oracle,
including moving meshes (velocity written, solid->fluid DDF reconstruction) and unvoxelization."""
import os

import numpy as np
import pytest

import oracle
import lbm_cases as LC
from fluidx3d_gb300 import LBM, TYPE_S, TYPE_X
from fluidx3d_gb300.mesh import ellipsoid_mesh

pytestmark = pytest.mark.gpu


def test_voxelize_matches_reference_fixture(gpu, golden_dir):
    g = np.load(os.path.join(golden_dir, "voxel.npz"))
    shape, mesh = LC.voxel_mesh_case()
    with LBM(*shape, 0.1) as lbm:
        lbm.voxelize_mesh_on_device(mesh, TYPE_S)
        assert np.array_equal(lbm.flags.data, g["flags"])


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "fp16c"])
def test_moving_mesh_matches_oracle(storage, gpu):
    shape = (40, 34, 30)
    o = oracle.Oracle(*shape, q=19, storage=storage, nu=0.05)
    o.initialize()
    with LBM(*shape, 0.05, storage=storage, arithmetic="exact") as lbm:
        lbm.run(0)  # initialise
        for k, shift in enumerate((0.0, 1.7)):
            mesh = ellipsoid_mesh(center=(17.0 + shift, 16.5, 14.2), semi_axes=(9.0, 7.5, 6.0), n_theta=16, n_phi=32, seed=3)
            lin, rot = (0.01, 0.0, 0.0), (0.0, 0.0, 0.01)
            lbm.voxelize_mesh_on_device(mesh, TYPE_S | TYPE_X, tuple(mesh.center), lin, rot)
            bbu, direction = LC.bbu_for(mesh, center=tuple(mesh.center), lin=lin, rot=rot)
            o.voxelize_mesh(direction, TYPE_S | TYPE_X, mesh.p0.reshape(-1), mesh.p1.reshape(-1), mesh.p2.reshape(-1), bbu, o.t + 1)
        lbm.flags.read_from_device()
        assert np.array_equal(lbm.flags.data, o.flags)
        assert np.array_equal(lbm.read_ddfs(), o.fi)
        lbm.run(3)
        o.run(3)
        assert np.array_equal(lbm.read_ddfs(), o.fi)
        mesh = ellipsoid_mesh(center=(18.7, 16.5, 14.2), semi_axes=(9.0, 7.5, 6.0), n_theta=16, n_phi=32, seed=3)
        lbm.unvoxelize_mesh_on_device(mesh, TYPE_X)
        o.unvoxelize_mesh(TYPE_X, *mesh.pmin, *mesh.pmax)
        lbm.flags.read_from_device()
        assert np.array_equal(lbm.flags.data, o.flags)


def test_large_mesh_voxelization_matches_oracle(gpu):
    """20k-triangle bumpy ellipsoid in a 160x96x96 box: flags bit-identical."""
    shape = (160, 96, 96)
    mesh = ellipsoid_mesh(center=(60.0, 48.3, 47.6), semi_axes=(50.0, 30.0, 30.0), n_theta=100, n_phi=100,
                          noise_amplitude=2.0, smooth_width=7, seed=11)
    o = oracle.Oracle(*shape, q=19, nu=0.1)
    bbu, direction = LC.bbu_for(mesh)
    o.voxelize_mesh(direction, TYPE_S, mesh.p0.reshape(-1), mesh.p1.reshape(-1), mesh.p2.reshape(-1), bbu, 1)
    with LBM(*shape, 0.1) as lbm:
        lbm.voxelize_mesh_on_device(mesh, TYPE_S)
        assert np.array_equal(lbm.flags.data, o.flags)
        assert int(np.sum(o.flags == TYPE_S)) > 100000
