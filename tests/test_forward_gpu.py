"""sm_103a forward kernels (initialize, stream_collide, update_fields, update_force_field) through the
C-ABI against the reference's golden fixtures and the FP32 CPU oracle: bit-identical results."""
import hashlib
import os

import numpy as np
import pytest

import oracle
import lbm_cases as LC
from fluidx3d_gb300 import LBM

pytestmark = pytest.mark.gpu


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_gpu(case):
    lbm = LBM(*case.shape, case.nu, *case.force, velocity_set=case.q, collision=case.collision, storage=case.storage,
              extensions=case.extensions)
    f = case.fields()
    lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:], lbm.F.data[:] = f["rho"], f["u"], f["flags"], f["F"]
    return lbm


def make_oracle(case):
    o = oracle.Oracle(*case.shape, q=case.q, collision=case.collision, storage=case.storage, extensions=case.extensions, nu=case.nu)
    f = case.fields()
    o.rho[:], o.u[:], o.flags[:], o.F[:] = f["rho"], f["u"], f["flags"], f["F"]
    return o


@pytest.mark.parametrize("case", LC.CASES, ids=[c.name for c in LC.CASES])
def test_gpu_matches_reference_fixture(case, gpu, golden_dir):
    g = np.load(os.path.join(golden_dir, f"lbm_{case.name}.npz"))
    with make_gpu(case) as lbm:
        lbm.run(case.steps)
        lbm.rho.read_from_device()
        lbm.u.read_from_device()
        assert np.array_equal(lbm.rho.data, g["rho"])
        assert np.array_equal(lbm.u.data, g["u"])
        assert sha(lbm.read_ddfs()) == str(g["fi_sha256"])
        if "ff" in case.extensions:
            lbm.update_force_field()
            lbm.F.read_from_device()
            assert np.array_equal(lbm.F.data, g["F"])


@pytest.mark.parametrize("case", LC.CASES, ids=[c.name for c in LC.CASES])
def test_gpu_matches_oracle_step_by_step(case, gpu):
    """DDFs after initialize and after 1, 2, 5 steps (both parities); fields at each stop."""
    o = make_oracle(case)
    with make_gpu(case) as lbm:
        o.initialize()
        lbm.initialize()
        assert np.array_equal(lbm.read_ddfs(), o.fi)
        lbm.u.read_from_device()
        assert np.array_equal(lbm.u.data, o.u)  # initialize zeroes u in solid cells
        for steps in (1, 1, 3):
            o.run(steps, *case.force)
            lbm.run(steps)
            assert lbm.get_t() == o.t
            assert np.array_equal(lbm.read_ddfs(), o.fi), f"DDFs differ at t={o.t}"
            o.update_fields(*case.force)
            lbm.rho.read_from_device()
            lbm.u.read_from_device()
            assert np.array_equal(lbm.rho.data, o.rho) and np.array_equal(lbm.u.data, o.u)


def test_taylor_green_64_bit_identical_to_reference(gpu, golden_dir):
    """64^3 TGV, D3Q19 SRT FP32, tau=0.6, 1000 steps: rho/u/DDF bytes equal the reference's."""
    g = np.load(os.path.join(golden_dir, "tgv64.npz"))
    case = LC.TGV64
    with make_gpu(case) as lbm:
        lbm.run(case.steps)
        lbm.rho.read_from_device()
        lbm.u.read_from_device()
        assert sha(lbm.rho.data) == str(g["rho_sha256"])
        assert sha(lbm.u.data) == str(g["u_sha256"])
        assert sha(lbm.read_ddfs()) == str(g["fi_sha256"])
        assert lbm.u.data[lbm.index(32, 32, 32)] == g["ux_center"]


def test_repeated_runs_are_deterministic(gpu):
    case = LC.CASE_BY_NAME["d3q19_trt_fp16s_channel_eq_ff_vf"]
    outs = []
    for _ in range(2):
        with make_gpu(case) as lbm:
            lbm.run(25)
            outs.append(lbm.read_ddfs())
    assert np.array_equal(*outs)


def test_run_in_chunks_equals_one_run(gpu):
    case = LC.CASE_BY_NAME["d3q19_srt_fp32_channel_eq_ff_vf"]
    with make_gpu(case) as a, make_gpu(case) as b:
        a.run(30)
        for k in (1, 7, 2, 20):
            b.run(k)
        assert a.get_t() == b.get_t() == 30
        assert np.array_equal(a.read_ddfs(), b.read_ddfs())


def test_set_force_between_steps(gpu):
    """The volume force can change between time steps (LBM::set_f) with the oracle agreeing."""
    case = LC.CASE_BY_NAME["d3q19_srt_fp32_tgv_vf"]
    o = make_oracle(case)
    with make_gpu(case) as lbm:
        o.initialize()
        lbm.run(3)
        o.run(3, *case.force)
        lbm.set_f(0.0, 2e-5, -1e-5)
        lbm.run(4)
        o.run(4, 0.0, 2e-5, -1e-5)
        assert np.array_equal(lbm.read_ddfs(), o.fi)
