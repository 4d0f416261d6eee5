"""lbm_object_sum_static (the allocation-free object reduction) against lbm_object_center_of_mass /
lbm_object_force / lbm_object_torque, both called through the C-ABI on the same device arrays.

The static variant reads the domain's own flags and F arrays (lbm_field_device_pointer) on the
domain's stream. With the default block count it sums in the same order as the domain calls; the
tests hold it to the FP64 reduction tolerance of the other object-sum tests (rtol 1e-12), on two
calls in a row, so a second call that reused stale scratch would show.
"""
import ctypes

import numpy as np
import pytest

from fluidx3d_gb300 import LBM, LBMError, TYPE_S, TYPE_X, _capi as C, setups as S

pytestmark = pytest.mark.gpu

MARKER = TYPE_S | TYPE_X
CENTER = (1.5, -0.25, 0.75)


@pytest.fixture(scope="module")
def domain(gpu):
    Nx, Ny, Nz = 64, 32, 32
    f = S.sphere_channel(Nx, Ny, Nz, u_in=0.05, radius=6.0, center=(20.0, 16.0, 16.0))
    lbm = LBM(Nx, Ny, Nz, 0.02, collision="trt", storage="fp32", extensions=("eq",), device=0)
    lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:] = f["rho"], f["u"], f["flags"]
    lbm.run(40)
    lbm.update_force_field()
    lbm.synchronize()
    yield lbm
    lbm.close()


def static_sum(lbm, kind, blocks=0, center=(0.0, 0.0, 0.0), F=None, marker=MARKER):
    flags_p, _ = lbm.device_pointer(C.FIELD_FLAGS)
    F_p = lbm.device_pointer(C.FIELD_F)[0] if F is None else F
    out = (ctypes.c_double * 4)()
    st = C.load().lbm_object_sum_static(0, lbm.get_Nx(), lbm.get_Ny(), lbm.get_Nz(), flags_p, F_p, marker, kind, *center, blocks, lbm.stream(), out)
    return st, np.array(out[:], dtype=np.float64)


def domain_sums(lbm):
    com, cells = lbm.object_center_of_mass(MARKER)
    return {0: np.array(list(com) + [cells], dtype=np.float64), 1: np.asarray(lbm.object_force(MARKER), dtype=np.float64),
            2: np.asarray(lbm.object_torque(CENTER, MARKER), dtype=np.float64)}


@pytest.mark.parametrize("blocks", [0, 1, 152, C.OBJECT_SUM_STATIC_MAX_BLOCKS])
def test_static_sum_matches_domain_calls_twice(domain, blocks):
    ref = domain_sums(domain)
    assert ref[0][3] > 100 and np.any(ref[1] != 0) and np.any(ref[2] != 0)
    for _ in range(2):  # two calls in a row
        for kind in (0, 1, 2):
            st, out = static_sum(domain, kind, blocks, CENTER if kind == 2 else (0.0, 0.0, 0.0))
            assert st == C.LBM_OK, C.load().lbm_last_error()
            n = 4 if kind == 0 else 3
            assert np.allclose(out[:n], ref[kind][:n], rtol=1e-12, atol=1e-13), (kind, blocks, out, ref[kind])
            if kind > 0:
                assert out[3] == 0.0


def test_static_sum_rejects_blocks_beyond_maximum(domain):
    st, _ = static_sum(domain, 1, C.OBJECT_SUM_STATIC_MAX_BLOCKS + 1)
    assert st == 1
    assert b"exceeds the static scratch maximum" in C.load().lbm_last_error()
    st, _ = static_sum(domain, 1, 0)  # the scratch still works after the rejected call
    assert st == C.LBM_OK


def test_static_sum_argument_errors(domain):
    st, _ = static_sum(domain, 3)
    assert st == 1
    flags_p, _ = domain.device_pointer(C.FIELD_FLAGS)
    out = (ctypes.c_double * 4)()
    assert C.load().lbm_object_sum_static(0, domain.get_Nx(), domain.get_Ny(), domain.get_Nz(), flags_p, None, MARKER, 1, 0.0, 0.0, 0.0, 0, None, out) == 1
    assert C.load().lbm_object_sum_static(0, 0, domain.get_Ny(), domain.get_Nz(), flags_p, None, MARKER, 0, 0.0, 0.0, 0.0, 0, None, out) == 1
    assert C.load().lbm_object_sum_static(-1, domain.get_Nx(), domain.get_Ny(), domain.get_Nz(), flags_p, None, MARKER, 0, 0.0, 0.0, 0.0, 0, None, out) == 1
