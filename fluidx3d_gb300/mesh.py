"""Triangle meshes for voxelization: the reference's ``struct Mesh`` (src/utilities.hpp:4440-4528),
its binary STL reader (src/utilities.hpp:4530-4581) and seeded procedural meshes.

Vertices are float32 arrays of shape (T, 3) in lattice coordinates (the box spans [0, N) per axis).
"""
from __future__ import annotations

import struct

import numpy as np


class Mesh:
    def __init__(self, p0, p1, p2, center=None):
        self.p0 = np.ascontiguousarray(p0, np.float32).reshape(-1, 3)
        self.p1 = np.ascontiguousarray(p1, np.float32).reshape(-1, 3)
        self.p2 = np.ascontiguousarray(p2, np.float32).reshape(-1, 3)
        self.find_bounds()
        self.center = np.asarray(center if center is not None else 0.5 * (self.pmin + self.pmax), np.float32)

    @property
    def triangle_number(self) -> int:
        return self.p0.shape[0]

    def find_bounds(self):
        allp = np.concatenate([self.p0, self.p1, self.p2])
        self.pmin = allp.min(axis=0).astype(np.float32)
        self.pmax = allp.max(axis=0).astype(np.float32)

    def translate(self, v):
        v = np.asarray(v, np.float32)
        self.p0 += v; self.p1 += v; self.p2 += v
        self.center = self.center + v
        self.pmin = self.pmin + v; self.pmax = self.pmax + v

    def scale(self, s):
        s = np.float32(s)
        for p in (self.p0, self.p1, self.p2):
            p[:] = s * (p - self.center) + self.center
        self.pmin = s * (self.pmin - self.center) + self.center
        self.pmax = s * (self.pmax - self.center) + self.center

    def rotate(self, R):
        R = np.asarray(R, np.float32)
        for p in (self.p0, self.p1, self.p2):
            p[:] = (p - self.center) @ R.T + self.center
        self.find_bounds()

    def bounding_box_size(self):
        return self.pmax - self.pmin


def read_stl(path, box_size=None, center=None, rotation=None, size=0.0, reposition=True) -> Mesh:
    """Binary STL (80-byte header, uint32 count, 50 bytes per triangle); rescaled and repositioned
    like read_stl_raw: size 0 fits the box, size > 0 sets the longest side, size < 0 scales by -size."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 84:
        raise ValueError(f"{path}: not a binary STL file")
    (T,) = struct.unpack_from("<I", data, 80)
    if T == 0 or len(data) != 84 + 50 * T:
        raise ValueError(f"{path}: corrupt or unsupported STL (only binary STL is supported)")
    rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")]), count=T, offset=84)
    v = rec["v"].astype(np.float32)
    R = np.eye(3, dtype=np.float32) if rotation is None else np.asarray(rotation, np.float32)

    def rot(q):  # float3x3*float3 in FP32, each row summed left to right
        return np.stack([(R[r, 0] * q[:, 0] + R[r, 1] * q[:, 1]) + R[r, 2] * q[:, 2] for r in range(3)], axis=1).astype(np.float32)
    p0, p1, p2 = rot(v[:, 0]), rot(v[:, 1]), rot(v[:, 2])
    allp = np.concatenate([p0, p1, p2])
    pmin, pmax = allp.min(axis=0), allp.max(axis=0)
    box = np.asarray(box_size if box_size is not None else (1.0, 1.0, 1.0), np.float32)
    c = np.asarray(center if center is not None else (0.0, 0.0, 0.0), np.float32)
    if size == 0.0:
        scale = float(np.min(box / (pmax - pmin)))
    elif size > 0.0:
        scale = size / float(np.max(pmax - pmin))
    else:
        scale = -size
    offset = -0.5 * (pmin + pmax) if reposition else np.zeros(3, np.float32)
    s = np.float32(scale)
    return Mesh(c + s * (offset + p0), c + s * (offset + p1), c + s * (offset + p2), center=c)


def write_stl(path, mesh: Mesh):
    T = mesh.triangle_number
    rec = np.zeros(T, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("attr", "<u2")]))
    rec["v"][:, 0], rec["v"][:, 1], rec["v"][:, 2] = mesh.p0, mesh.p1, mesh.p2
    with open(path, "wb") as f:
        f.write(b"\0" * 80 + struct.pack("<I", T) + rec.tobytes())


def _periodic_box_smooth(a, width, axis):
    acc = np.zeros_like(a)
    for s in range(-(width // 2), width // 2 + 1):
        acc += np.roll(a, s, axis=axis)
    return acc / width


def ellipsoid_mesh(center, semi_axes, n_theta=64, n_phi=128, noise_amplitude=0.0, smooth_width=9, seed=0) -> Mesh:
    """Closed, outward-oriented UV ellipsoid of 2*n_phi*(n_theta-1) triangles. With noise, the radius
    of every vertex is scaled by (1 + noise/r_mean), noise = seeded uniform [-a, a] on the
    (theta, phi) vertex grid smoothed by a box filter (periodic in phi) and rescaled to amplitude a."""
    rng = np.random.default_rng(seed)
    th = np.linspace(0.0, np.pi, n_theta + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, n_phi, endpoint=False)
    TH, PH = np.meshgrid(th, ph, indexing="ij")
    a = np.asarray(semi_axes, np.float64)
    dirs = np.stack([np.sin(TH) * np.cos(PH), np.sin(TH) * np.sin(PH), np.cos(TH)], axis=-1)
    scale = np.ones(TH.shape)
    if noise_amplitude > 0.0:
        noise = rng.uniform(-1.0, 1.0, TH.shape)
        noise = _periodic_box_smooth(noise, smooth_width, axis=1)
        noise = _periodic_box_smooth(np.pad(noise, ((smooth_width, smooth_width), (0, 0)), mode="edge"), smooth_width, axis=0)[smooth_width:-smooth_width]
        noise *= noise_amplitude / max(np.max(np.abs(noise)), 1e-30)
        noise[0, :] = noise[0, :].mean()  # poles: one radius per pole
        noise[-1, :] = noise[-1, :].mean()
        scale = 1.0 + noise / a.mean()
    V = np.asarray(center, np.float64) + dirs * a * scale[..., None]
    tris = []
    for i in range(n_theta):
        j = np.arange(n_phi)
        jn = (j + 1) % n_phi
        A, B, Cc, D = V[i, j], V[i, jn], V[i + 1, j], V[i + 1, jn]
        if i > 0:
            tris.append(np.stack([A, Cc, B], axis=1))
        if i < n_theta - 1:
            tris.append(np.stack([B, Cc, D], axis=1))
    t = np.concatenate(tris).astype(np.float32)
    return Mesh(t[:, 0], t[:, 1], t[:, 2], center=np.asarray(center, np.float32))


def sphere_mesh(center, radius, n_theta=32, n_phi=64) -> Mesh:
    return ellipsoid_mesh(center, (radius, radius, radius), n_theta, n_phi)
