"""Parity cases shared by the golden-fixture generator and the tests.

Each case is one variant of the reference's compile-time switches (velocity set, collision
operator, DDF storage, extensions) on a small seeded geometry, small enough for the CPU oracle to
finish in well under a second.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from fluidx3d_gb300 import setups as S


@dataclass(frozen=True)
class Case:
    name: str
    q: int
    collision: str
    storage: str
    extensions: tuple = ()
    geometry: str = "tgv"        # "tgv" | "channel" | "cavity" | "couette"
    shape: tuple = (16, 12, 10)
    nu: float = 0.04
    steps: int = 37
    fx: float = 0.0
    seed: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def N(self):
        return self.shape[0] * self.shape[1] * self.shape[2]

    def fields(self):
        Nx, Ny, Nz = self.shape
        if self.geometry == "tgv":
            c = S.taylor_green(Nx, Ny, Nz)
        elif self.geometry == "cavity":
            c = S.lid_driven_cavity(Nx, Ny, Nz, u_lid=0.1)
        elif self.geometry == "couette":
            c = S.taylor_couette(Nx, Ny, Nz, seed=self.seed)
        else:
            c = S.sphere_channel(Nx, Ny, Nz, u_in=0.05, radius=3.0, center=(Nx / 3.0, Ny / 2.0, Nz / 2.0))
            if "sphere_u" in self.extra:  # a moving sphere (MOVING_BOUNDARIES)
                N = self.N
                sphere = (c["flags"] & S.TYPE_X) != 0
                for d, v in enumerate(self.extra["sphere_u"]):
                    c["u"][d * N:(d + 1) * N][sphere] = np.float32(v)
        if "ff" in self.extensions:
            rng = np.random.default_rng(self.seed)
            c["F"] = rng.normal(0.0, 1e-4, 3 * self.N).astype(np.float32)
        return c

    @property
    def force(self):
        return (self.fx, 0.0, 0.0)

    def settle_fields(self, m):
        """rho/u as a read of the fields gives them: update_fields, except with UPDATE_FIELDS, where
        the steps wrote them (the fields of the state each step started from) and update_fields is
        compiled out (src/lbm.cpp:184-191)."""
        if "uf" not in self.extensions:
            m.update_fields(*self.force)


CASES = [
    Case("d3q19_srt_fp32_tgv", 19, "srt", "fp32"),
    Case("d3q19_srt_fp16s_tgv", 19, "srt", "fp16s"),
    Case("d3q19_srt_fp16c_tgv", 19, "srt", "fp16c"),
    Case("d3q19_trt_fp32_tgv", 19, "trt", "fp32"),
    Case("d3q19_trt_fp16s_channel_eq_ff_vf", 19, "trt", "fp16s", ("eq", "ff", "vf"), "channel", fx=1e-5),
    Case("d3q19_srt_fp32_channel_eq_ff_vf", 19, "srt", "fp32", ("eq", "ff", "vf"), "channel", fx=1e-5),
    Case("d3q19_trt_fp32_channel_eq_ff_vf", 19, "trt", "fp32", ("eq", "ff", "vf"), "channel", fx=1e-5),
    Case("d3q19_srt_fp32_tgv_vf", 19, "srt", "fp32", ("vf",), fx=1e-5),
    Case("d3q19_srt_fp16c_channel_eq", 19, "srt", "fp16c", ("eq",), "channel"),
    Case("d3q27_srt_fp32_tgv", 27, "srt", "fp32"),
    Case("d3q27_trt_fp32_channel_eq_ff_vf", 27, "trt", "fp32", ("eq", "ff", "vf"), "channel", fx=1e-5),
    Case("d3q27_srt_fp16s_tgv", 27, "srt", "fp16s"),
    Case("d3q19_srt_fp32_tgv_sg", 19, "srt", "fp32", ("sg",)),
    Case("d3q19_trt_fp16s_channel_eq_sg", 19, "trt", "fp16s", ("eq", "sg"), "channel"),
    Case("d3q27_trt_fp32_channel_eq_ff_sg_vf", 27, "trt", "fp32", ("eq", "ff", "sg", "vf"), "channel", fx=1e-5),
    Case("d3q19_srt_fp32_cavity_mb", 19, "srt", "fp32", ("mb",), "cavity"),
    Case("d3q19_trt_fp16s_couette_mb", 19, "trt", "fp16s", ("mb",), "couette", (16, 16, 12)),
    Case("d3q19_trt_fp16c_couette_mb_sg", 19, "trt", "fp16c", ("mb", "sg"), "couette", (16, 16, 12), nu=0.01),
    Case("d3q27_trt_fp32_channel_eq_ff_mb_vf", 27, "trt", "fp32", ("eq", "ff", "mb", "vf"), "channel", fx=1e-5,
         extra={"sphere_u": (0.0, 0.02, -0.01)}),
    Case("d3q19_srt_fp32_tgv_uf", 19, "srt", "fp32", ("uf",)),
    Case("d3q19_trt_fp16s_channel_eq_ff_uf_vf", 19, "trt", "fp16s", ("eq", "ff", "uf", "vf"), "channel", fx=1e-5),
    Case("d3q27_trt_fp16c_couette_eq_mb_uf", 27, "trt", "fp16c", ("eq", "mb", "uf"), "couette", (16, 16, 12)),
]
CASE_BY_NAME = {c.name: c for c in CASES}

# the Taylor-Green workload at full size: 64^3, D3Q19 SRT FP32, tau = 0.6 (nu = 1/30), 1000 steps
TGV64 = Case("tgv64_d3q19_srt_fp32", 19, "srt", "fp32", (), "tgv", (64, 64, 64), nu=1.0 / 30.0, steps=1000)


def voxel_mesh_case():
    """A seeded bumpy ellipsoid inside a 48x40x36 box, for bit-exact flag parity."""
    from fluidx3d_gb300.mesh import ellipsoid_mesh
    shape = (48, 40, 36)
    mesh = ellipsoid_mesh(center=(21.3, 19.7, 17.9), semi_axes=(14.2, 11.1, 9.6), n_theta=24, n_phi=48,
                          noise_amplitude=1.5, smooth_width=5, seed=7)
    return shape, mesh


def bbu_for(mesh, center=(0.0, 0.0, 0.0), lin=(0.0, 0.0, 0.0), rot=(0.0, 0.0, 0.0)):
    """16-float bounding-box/velocity block and ray direction exactly as the reference's host code
    builds them (src/lbm.cpp:280-318); used to drive the CPU libraries directly."""
    pmin, pmax = mesh.pmin.astype(np.float32), mesh.pmax.astype(np.float32)
    two = np.float32(2.0)
    x0, y0, z0 = pmin - two
    x1, y1, z1 = pmax + two
    bbu = np.zeros(16, np.float32)
    bbu[0] = np.array([mesh.triangle_number], np.uint32).view(np.float32)[0]
    bbu[1:7] = [x0, y0, z0, x1, y1, z1]
    bbu[7:10], bbu[10:13], bbu[13:16] = center, lin, rot
    rv = np.asarray(rot, np.float32)
    if float(np.sqrt(np.sum(rv * rv))) == 0.0:
        v = np.array([(y1 - y0) * (z1 - z0), (z1 - z0) * (x1 - x0), (x1 - x0) * (y1 - y0)], np.float32)
        direction = 0
        for i in (1, 2):
            if v[i] < v[direction]:
                direction = i
    else:
        direction = int(np.argmax(np.abs(rv)))
    return bbu, direction
