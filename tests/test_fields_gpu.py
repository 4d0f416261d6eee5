"""Force field, FP64 object reductions and the lazy field/force bookkeeping on the GPU."""
import numpy as np
import pytest

import oracle
import lbm_cases as LC
from fluidx3d_gb300 import LBM, LBMError, TYPE_S, TYPE_X
from test_forward_gpu import make_gpu, make_oracle

pytestmark = pytest.mark.gpu


def _run_both(case, steps):
    o = make_oracle(case)
    o.initialize()
    o.run(steps, *case.force)
    o.update_force_field()
    lbm = make_gpu(case)
    lbm.run(steps)
    return o, lbm


@pytest.mark.parametrize("name", ["d3q19_trt_fp16s_channel_eq_ff_vf", "d3q27_trt_fp32_channel_eq_ff_vf", "d3q19_srt_fp16c_channel_eq"])
def test_force_torque_com_fp64(name, gpu):
    case = LC.CASE_BY_NAME[name]
    o, lbm = _run_both(case, 21)
    with lbm:
        lbm.update_force_field()
        lbm.F.read_from_device()
        solid = (lbm.flags.data & 3) == 1
        assert np.array_equal(np.where(np.tile(solid, 3), lbm.F.data, 0), np.where(np.tile(solid, 3), o.F, 0))
        marker = TYPE_S | TYPE_X
        F = lbm.object_force(marker)
        ref = o.object_sum(1, marker)
        assert np.allclose(F, ref[:3], rtol=1e-12, atol=1e-15) and np.any(F != 0)
        c = (1.5, -0.25, 0.75)
        T = lbm.object_torque(c, marker)
        assert np.allclose(T, o.object_sum(2, marker, c)[:3], rtol=1e-12, atol=1e-15)
        com, cells = lbm.object_center_of_mass(marker)
        s = o.object_sum(0, marker)
        assert cells == int(s[3]) > 50 and np.allclose(com, s[:3] / s[3], rtol=1e-12, atol=1e-12)


def test_lazy_update_fields_and_force(gpu):
    case = LC.CASE_BY_NAME["d3q19_srt_fp32_channel_eq_ff_vf"]
    with make_gpu(case) as lbm:
        lbm.run(5)
        lbm.u.read_from_device()
        u1 = lbm.u.data.copy()
        lbm.u.data[:] = 7.0  # host edits without a step: reading again returns device data
        lbm.u.read_from_device()
        assert np.array_equal(lbm.u.data, u1)
        lbm.run(1)
        lbm.u.read_from_device()
        assert not np.array_equal(lbm.u.data, u1)
        f1 = lbm.object_force(TYPE_S | TYPE_X)
        f2 = lbm.object_force(TYPE_S | TYPE_X)
        assert np.array_equal(f1, f2)


def test_force_field_without_extension_allocates_on_demand(gpu):
    """update_force_field also works without FORCE_FIELD (drag on obstacles without a force input)."""
    case = LC.CASE_BY_NAME["d3q19_srt_fp16c_channel_eq"]
    o, lbm = _run_both(case, 9)
    with lbm:
        with pytest.raises(LBMError):
            lbm.F.read_from_device()  # F does not exist yet
        lbm.update_force_field()
        lbm.F.read_from_device()
        solid = np.tile((lbm.flags.data & 3) == 1, 3)
        assert np.array_equal(lbm.F.data[solid], o.F[solid])


def test_errors_are_reported_not_fatal(gpu):
    with LBM(8, 8, 8, 0.1) as lbm:
        with pytest.raises(LBMError) as e:
            lbm.update_fields()
        assert e.value.status == 4  # not initialised
        with pytest.raises(LBMError) as e:
            lbm.set_f(1e-5, 0, 0)  # no VOLUME_FORCE
        assert e.value.status == 5
        import ctypes
        from fluidx3d_gb300 import _capi as C
        buf = np.zeros(10, np.float32)
        assert C.load().lbm_write_field(lbm.handle, C.FIELD_RHO, buf.ctypes.data, buf.nbytes) == 1
        assert C.load().lbm_write_field(lbm.handle, 99, buf.ctypes.data, buf.nbytes) == 1
        assert b"bytes" in C.load().lbm_last_error() or b"field" in C.load().lbm_last_error()
        lbm.run(3)  # the domain stays usable
        assert lbm.get_t() == 3


@pytest.mark.parametrize("arithmetic,path", [("exact", "cells"), ("fast", "cells"), ("fast", "pipe"), ("fast", "pairs")])
def test_fused_update_fields_lag_one_step(arithmetic, path, gpu, monkeypatch):
    """UPDATE_FIELDS: after run(k) rho/u are the fields of the state at t = k-1, bit for bit what
    update_fields gives after run(k-1) without the extension (TYPE_E cells keep their preset values);
    update_fields is a no-op; the reference's byte accounting adds 16 B per cell."""
    monkeypatch.setenv("FX3D_STREAM_COLLIDE_PATH", path)
    base = LC.CASE_BY_NAME["d3q19_trt_fp16s_channel_eq_ff_vf"]
    fused_case = LC.Case("fused", base.q, base.collision, base.storage, base.extensions + ("uf",), base.geometry, fx=base.fx)
    with make_gpu(base, arithmetic) as plain, make_gpu(fused_case, arithmetic) as fused:
        plain.run(6)
        plain.update_fields()
        fused.run(7)
        for lbm in (plain, fused):
            lbm.rho.read_from_device()
            lbm.u.read_from_device()
        assert np.array_equal(fused.rho.data, plain.rho.data)
        assert np.array_equal(fused.u.data, plain.u.data)
        fused.update_fields()
        fused.u.read_from_device()
        assert np.array_equal(fused.u.data, plain.u.data)
        assert fused.bandwidth_bytes_per_cell() == plain.bandwidth_bytes_per_cell() + 16
