"""The GPU adjoint (FP32, checkpointed) against the FP64 discrete adjoint of the CPU oracle, which is
itself checked against central finite differences in tests/test_adjoint_oracle.py."""
import numpy as np
import pytest

import oracle
from fluidx3d_gb300 import LBM, setups as S
from test_adjoint_oracle import channel_problem

pytestmark = pytest.mark.gpu


def gpu_problem(collision, storage="fp32", Nx=24, Ny=12, Nz=12, seed=3, q=19):
    f = S.sphere_channel(Nx, Ny, Nz, u_in=0.05, radius=2.5, center=(8.0, 6.0, 6.0))
    F = S.box_filter_noise(Nx, Ny, Nz, sigma=1e-4, width=3, seed=seed)
    lbm = LBM(Nx, Ny, Nz, 0.02, 2e-6, 0.0, 0.0, velocity_set=q, collision=collision, storage=storage, extensions=("eq", "ff", "vf"))
    lbm.rho.data[:], lbm.u.data[:], lbm.flags.data[:], lbm.F.data[:] = f["rho"], f["u"], f["flags"], F
    return lbm


@pytest.mark.parametrize("collision,kind,q", [("srt", "ke_plane", 19), ("trt", "ke_plane", 19), ("trt", "drag_x", 19), ("srt", "drag_x", 19),
                                              ("trt", "ke_plane", 27), ("srt", "drag_x", 27)])
def test_gpu_adjoint_matches_fp64_adjoint(collision, kind, q, gpu):
    o, f0 = channel_problem(collision, q=q)
    obj = oracle.objective(kind, 28, 40, plane_x=18, marker=0x41)
    J64, g64 = oracle.fp64_adjoint(o, f0, 40, obj, interval=7, force=(2e-6, 0.0, 0.0))
    with gpu_problem(collision, q=q) as lbm:
        J, g, stats = lbm.run_adjoint(40, kind, window=(28, 40), plane_x=18, marker=0x41, checkpoint_interval=7)
        assert lbm.get_t() == 40
    assert J == pytest.approx(J64, rel=2e-5)
    scale = np.max(np.abs(g64))
    assert scale > 0
    assert np.max(np.abs(g - g64)) <= 1e-3 * scale, np.max(np.abs(g - g64)) / scale


def test_gpu_adjoint_checkpointing_is_exact(gpu):
    """Gradients do not depend on the checkpoint interval (recomputed states are bit-identical)."""
    outs = []
    for interval in (1, 6, 40):
        with gpu_problem("trt") as lbm:
            outs.append(lbm.run_adjoint(40, "ke_plane", window=(20, 40), plane_x=18, checkpoint_interval=interval)[:2])
    for J, g in outs[1:]:
        assert J == outs[0][0] and np.array_equal(g, outs[0][1])


def test_gpu_adjoint_leaves_the_forward_state(gpu):
    with gpu_problem("trt") as a, gpu_problem("trt") as b:
        a.run_adjoint(25, "drag_x", window=(10, 25), marker=0x41, checkpoint_interval=4)
        b.run(25)
        assert a.get_t() == b.get_t() == 25
        assert np.array_equal(a.read_ddfs(), b.read_ddfs())


def test_gpu_adjoint_fp16s_storage_close_to_fp32(gpu):
    """FP16S-stored DDFs (and snapshots): gradient within 2% of the FP32-storage gradient."""
    res = []
    for storage in ("fp32", "fp16s"):
        with gpu_problem("trt", storage) as lbm:
            res.append(lbm.run_adjoint(40, "ke_plane", window=(28, 40), plane_x=18, checkpoint_interval=8)[1])
    scale = np.max(np.abs(res[0]))
    assert np.max(np.abs(res[1] - res[0])) <= 2e-2 * scale


def test_autograd_shim_gives_the_adjoint_gradient(gpu):
    torch = pytest.importorskip("torch")
    from adjoint_autograd import LBMObjective
    base = gpu_problem("trt")
    F0 = base.F.data.copy()
    base.close()
    F = torch.tensor(F0, dtype=torch.float32, requires_grad=True)
    kw = dict(steps=30, objective="ke_plane", window=(20, 30), plane_x=18, checkpoint_interval=10)
    J = LBMObjective.apply(F, lambda: gpu_problem("trt"), kw)
    (g,) = torch.autograd.grad(J, F)
    with gpu_problem("trt") as lbm:
        J2, g2, _ = lbm.run_adjoint(**kw)
    assert float(J) == J2 and np.array_equal(g.numpy(), g2)
    # directional derivative against a central difference of the GPU forward objective (FP32, large step)
    d = np.random.default_rng(0).normal(0, 1, F0.size).astype(np.float32) * np.float32(np.abs(F0).max())
    h = 0.5  # the objective is close to quadratic in the small force field: a large step is accurate
    Jp = float(LBMObjective.apply(torch.tensor(F0 + h * d), lambda: gpu_problem("trt"), kw))
    Jm = float(LBMObjective.apply(torch.tensor(F0 - h * d), lambda: gpu_problem("trt"), kw))
    fd = (Jp - Jm) / (2 * h)
    ad = float(np.dot(g2.astype(np.float64), d.astype(np.float64)))
    assert abs(fd - ad) <= 2e-2 * abs(ad), (fd, ad)


def test_gpu_adjoint_workspace_plans_give_the_same_gradient(gpu):
    """A workspace limit selects the plan: two moment sets with overlapped recomputation, one set
    without overlap, or two levels of DDF sub-snapshots. Every plan recomputes the same states and
    moments, so J and dJ/dF are bit-identical; too small a limit is an out-of-memory error.
    Workspace of the 24x12x12 FP32 D3Q19 problem (N = 3456): DDF state 262,656 B, moments of a step
    55,296 B, lambda + gradient 304,192 B; 40 steps with interval 20: overlapped 3,304,000 B, one set
    2,198,080 B; interval 40 (one segment): one set 3,041,344 B, two levels (K2 = 7) 2,792,512 B."""
    from fluidx3d_gb300._capi import LBMError
    kw = dict(window=(20, 40), plane_x=18)
    plans = [(20, 0, dict(levels=1, overlapped=1)), (20, 3000, dict(levels=1, overlapped=0)), (40, 2900, dict(levels=2, overlapped=0))]
    outs = []
    for interval, limit, expect in plans:
        with gpu_problem("trt") as lbm:
            J, g, st = lbm.run_adjoint(40, "ke_plane", checkpoint_interval=interval, workspace_limit_kib=limit, **kw)
        assert {k: st[k] for k in expect} == expect, (interval, limit, st)
        outs.append((J, g))
    for J, g in outs[1:]:
        assert J == outs[0][0] and np.array_equal(g, outs[0][1])
    with gpu_problem("trt") as lbm:
        with pytest.raises(LBMError, match="workspace"):
            lbm.run_adjoint(40, "ke_plane", checkpoint_interval=20, workspace_limit_kib=1000, **kw)
