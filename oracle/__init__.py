"""CPU oracle for the LBM solver path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import this package,
and only as the checker or the timed CPU baseline. The product package ``fluidx3d_gb300`` never
imports it.

Two CPU libraries are wrapped here:
  * ``Oracle``: oracle/lbm_oracle.cpp, a restatement of the reference's scheme (FP32 op-for-op and
    FP64), built into oracle/_build/;
  * ``RefHarness``: the reference's own OpenCL C kernel text compiled for the CPU
    (oracle/ref_harness, built into oracle/_ref/ only where the reference text is available).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblbm_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

STORAGE = {"fp32": 0, "fp16s": 1, "fp16c": 2}
EXT_BITS = {"vf": 1, "ff": 2, "eq": 4, "sg": 8, "mb": 16, "uf": 32}


def build_oracle(force: bool = False) -> str:
    src = [os.path.join(HERE, "lbm_oracle.cpp"), os.path.join(HERE, "half_ieee.h")]
    if not force and os.path.isfile(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".{os.getpid()}.tmp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
                    src[0], "-o", tmp], check=True)
    os.replace(tmp, LIB)
    return LIB


class OracleConfig(ctypes.Structure):
    _fields_ = [("Nx", ctypes.c_uint32), ("Ny", ctypes.c_uint32), ("Nz", ctypes.c_uint32),
                ("q", ctypes.c_uint32), ("trt", ctypes.c_uint32), ("storage", ctypes.c_uint32),
                ("ext", ctypes.c_uint32), ("threads", ctypes.c_uint32), ("w", ctypes.c_double)]


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build_oracle())
        v, f32, f64, u8, u16, u32, u64, d = (ctypes.c_void_p, ctypes.c_float, ctypes.c_double, ctypes.c_uint8,
                                             ctypes.c_uint16, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double)
        cfg = ctypes.POINTER(OracleConfig)
        L.oracle_kernel_w.argtypes = [f32]; L.oracle_kernel_w.restype = f32
        for s, r in (("f32", f32), ("f64", f64)):
            getattr(L, f"oracle_initialize_{s}").argtypes = [cfg, v, v, v, v]
            getattr(L, f"oracle_stream_collide_{s}").argtypes = [cfg, v, v, v, v, u64, r, r, r, v]
            getattr(L, f"oracle_run_{s}").argtypes = [cfg, v, v, v, v, u64, u64, r, r, r, v]
            getattr(L, f"oracle_update_fields_{s}").argtypes = [cfg, v, v, v, v, u64, r, r, r, v]
            getattr(L, f"oracle_update_force_field_{s}").argtypes = [cfg, v, v, u64, v]
            getattr(L, f"oracle_update_moving_boundaries_{s}").argtypes = [cfg, v, v]
        L.oracle_object_sum.argtypes = [cfg, ctypes.c_int, v, v, u8, d, d, d, v]
        L.oracle_voxelize_mesh.argtypes = [cfg, u32, v, v, v, u64, u8, v, v, v, v]
        L.oracle_voxelize_rays.argtypes = [cfg, u32, v, v, v, u64, u8, v, v, v, v, v, u64]
        L.oracle_unvoxelize_mesh.argtypes = [cfg, v, u8, f32, f32, f32, f32, f32, f32]
        L.oracle_fp16s_encode.argtypes = [f32]; L.oracle_fp16s_encode.restype = u16
        L.oracle_fp16s_decode.argtypes = [u16]; L.oracle_fp16s_decode.restype = f32
        L.oracle_fp16c_encode.argtypes = [f32]; L.oracle_fp16c_encode.restype = u16
        L.oracle_fp16c_decode.argtypes = [u16]; L.oracle_fp16c_decode.restype = f32
        _lib = L
    return _lib


def kernel_w(nu: float) -> float:
    """Relaxation rate as the reference bakes it into its kernel (1/tau printed with "%f")."""
    return float(lib().oracle_kernel_w(nu))


def ext_bits(extensions) -> int:
    return sum(EXT_BITS[e] for e in set(extensions))


class Oracle:
    """One LBM domain on the CPU in FP32 (``precision="f32"``) or FP64 (``"f64"``).

    Arrays follow the reference's layout: fi is q*N (SoA, fi[i*N+n]), rho N, u 3*N (SoA), flags N
    uint8, F 3*N. In f32 mode fi has the storage dtype (float32, or uint16 for FP16S/FP16C).
    """

    def __init__(self, Nx, Ny, Nz, q=19, collision="srt", storage="fp32", extensions=(), w=None, nu=None,
                 precision="f32", threads=None):
        self.Nx, self.Ny, self.Nz, self.q = int(Nx), int(Ny), int(Nz), int(q)
        self.N = self.Nx * self.Ny * self.Nz
        self.precision = precision
        self.storage = storage if precision == "f32" else "fp32"
        if w is None:
            w = kernel_w(nu)
        self.w = float(w)
        self.cfg = OracleConfig(self.Nx, self.Ny, self.Nz, self.q, 1 if collision == "trt" else 0,
                                STORAGE[self.storage], ext_bits(extensions), threads or os.cpu_count() or 1, self.w)
        self.real = np.float32 if precision == "f32" else np.float64
        ddf_dtype = self.real if self.storage == "fp32" else np.uint16
        self.fi = np.zeros(self.q * self.N, dtype=ddf_dtype)
        self.rho = np.ones(self.N, dtype=self.real)
        self.u = np.zeros(3 * self.N, dtype=self.real)
        self.flags = np.zeros(self.N, dtype=np.uint8)
        self.F = np.zeros(3 * self.N, dtype=self.real)
        self.t = 0

    def _fn(self, name):
        return getattr(lib(), f"oracle_{name}_{self.precision}")

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"oracle {what} failed ({rc})")

    def initialize(self):
        self._chk(self._fn("initialize")(ctypes.byref(self.cfg), _p(self.fi), _p(self.rho), _p(self.u), _p(self.flags)), "initialize")
        self.t = 0

    def run(self, steps, fx=0.0, fy=0.0, fz=0.0):
        self._chk(self._fn("run")(ctypes.byref(self.cfg), _p(self.fi), _p(self.rho), _p(self.u), _p(self.flags), self.t, steps,
                                  fx, fy, fz, _p(self.F)), "run")
        self.t += steps

    def update_fields(self, fx=0.0, fy=0.0, fz=0.0):
        self._chk(self._fn("update_fields")(ctypes.byref(self.cfg), _p(self.fi), _p(self.rho), _p(self.u), _p(self.flags), self.t,
                                            fx, fy, fz, _p(self.F)), "update_fields")

    def update_force_field(self):
        self._chk(self._fn("update_force_field")(ctypes.byref(self.cfg), _p(self.fi), _p(self.flags), self.t, _p(self.F)),
                  "update_force_field")

    def update_moving_boundaries(self):
        self._chk(self._fn("update_moving_boundaries")(ctypes.byref(self.cfg), _p(self.u), _p(self.flags)), "update_moving_boundaries")

    def object_sum(self, kind, marker, center=(0.0, 0.0, 0.0)):
        out = np.zeros(4, dtype=np.float64)
        F = np.ascontiguousarray(self.F, dtype=np.float32)
        self._chk(lib().oracle_object_sum(ctypes.byref(self.cfg), kind, _p(F), _p(self.flags), marker, *center, _p(out)), "object_sum")
        return out

    def voxelize_mesh(self, direction, flag, p0, p1, p2, bbu, t):
        assert self.precision == "f32"
        self._chk(lib().oracle_voxelize_mesh(ctypes.byref(self.cfg), direction, _p(self.fi), _p(self.u), _p(self.flags), t, flag,
                                             _p(p0), _p(p1), _p(p2), _p(bbu)), "voxelize_mesh")

    def unvoxelize_mesh(self, flag, x0, y0, z0, x1, y1, z1):
        self._chk(lib().oracle_unvoxelize_mesh(ctypes.byref(self.cfg), _p(self.flags), flag, x0, y0, z0, x1, y1, z1), "unvoxelize_mesh")


def voxelize_rays(shape, flags, direction, flag, p0, p1, p2, bbu, rays, q=19, threads=None):
    """The FP32 voxelizer restatement (src/kernel.cpp:2267-2357) on a subset of rays only, into a
    flags array of the whole lattice (no DDFs or velocities: for a mesh without velocity over cells
    that start without the mesh's flag). Ray index a as the kernel's: direction 0 a = y + z*Ny,
    1 a = z + x*Nz, 2 a = x + y*Nx."""
    Nx, Ny, Nz = (int(v) for v in shape)
    assert flags.dtype == np.uint8 and flags.size == Nx * Ny * Nz
    assert not np.any(np.asarray(bbu[7:16], np.float32)[3:] != 0.0), "mesh velocity needs DDFs and u"
    cfg = OracleConfig(Nx, Ny, Nz, q, 0, STORAGE["fp32"], 0, threads or os.cpu_count() or 1, 1.0)
    rays = np.ascontiguousarray(rays, dtype=np.uint64)
    rc = lib().oracle_voxelize_rays(ctypes.byref(cfg), direction, None, None, _p(flags), 0, flag, _p(np.ascontiguousarray(p0, np.float32)),
                                    _p(np.ascontiguousarray(p1, np.float32)), _p(np.ascontiguousarray(p2, np.float32)),
                                    _p(np.ascontiguousarray(bbu, np.float32)), _p(rays), rays.size)
    if rc != 0:
        raise RuntimeError(f"oracle voxelize_rays failed ({rc})")


def ref_variant_name(q, collision, storage, extensions=()) -> str:
    ext = "".join("_" + e for e in sorted(set(extensions)))
    return f"d3q{q}_{collision}_{storage}{ext}"


def ref_available(q=19, collision="srt", storage="fp32", extensions=()) -> bool:
    return os.path.isfile(os.path.join(REF_DIR, f"ref_{ref_variant_name(q, collision, storage, extensions)}.so"))


class RefHarness:
    """The reference's own kernels (compiled for the CPU) over numpy arrays in the reference layout."""

    def __init__(self, Nx, Ny, Nz, q=19, collision="srt", storage="fp32", extensions=(), w=None, nu=None, threads=None):
        path = os.path.join(REF_DIR, f"ref_{ref_variant_name(q, collision, storage, extensions)}.so")
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        v, f32, u8, u32, u64 = ctypes.c_void_p, ctypes.c_float, ctypes.c_uint8, ctypes.c_uint32, ctypes.c_uint64
        L.ref_configure.argtypes = [u32, u32, u32, f32, u32]
        L.ref_initialize.argtypes = [v, v, v, v]
        L.ref_stream_collide.argtypes = [v, v, v, v, u64, f32, f32, f32, v]
        L.ref_update_fields.argtypes = [v, v, v, v, u64, f32, f32, f32, v]
        L.ref_update_force_field.argtypes = [v, v, u64, v]
        L.ref_update_moving_boundaries.argtypes = [v, v]
        L.ref_voxelize_mesh.argtypes = [u32, v, v, v, u64, u8, v, v, v, v]
        L.ref_unvoxelize_mesh.argtypes = [v, u8, f32, f32, f32, f32, f32, f32]
        self.L = L
        self.Nx, self.Ny, self.Nz, self.q = int(Nx), int(Ny), int(Nz), int(q)
        self.N = self.Nx * self.Ny * self.Nz
        self.w = float(kernel_w(nu) if w is None else w)
        self.threads = threads or os.cpu_count() or 1
        self.fi = np.zeros(self.q * self.N, dtype=np.float32 if storage == "fp32" else np.uint16)
        self.rho = np.ones(self.N, dtype=np.float32)
        self.u = np.zeros(3 * self.N, dtype=np.float32)
        self.flags = np.zeros(self.N, dtype=np.uint8)
        self.F = np.zeros(3 * self.N, dtype=np.float32)
        self.t = 0

    def _cfg(self):
        self.L.ref_configure(self.Nx, self.Ny, self.Nz, self.w, self.threads)

    def initialize(self):
        self._cfg()
        self.L.ref_initialize(_p(self.fi), _p(self.rho), _p(self.u), _p(self.flags))
        self.t = 0

    def run(self, steps, fx=0.0, fy=0.0, fz=0.0):
        self._cfg()
        for _ in range(steps):
            self.L.ref_stream_collide(_p(self.fi), _p(self.rho), _p(self.u), _p(self.flags), self.t, fx, fy, fz, _p(self.F))
            self.t += 1

    def update_fields(self, fx=0.0, fy=0.0, fz=0.0):
        self._cfg()
        self.L.ref_update_fields(_p(self.fi), _p(self.rho), _p(self.u), _p(self.flags), self.t, fx, fy, fz, _p(self.F))

    def update_force_field(self):
        self._cfg()
        if self.L.ref_update_force_field(_p(self.fi), _p(self.flags), self.t, _p(self.F)) != 0:
            raise RuntimeError("update_force_field needs the FORCE_FIELD variant")

    def update_moving_boundaries(self):
        self._cfg()
        if self.L.ref_update_moving_boundaries(_p(self.u), _p(self.flags)) != 0:
            raise RuntimeError("update_moving_boundaries needs the MOVING_BOUNDARIES variant")

    def voxelize_mesh(self, direction, flag, p0, p1, p2, bbu, t):
        self._cfg()
        self.L.ref_voxelize_mesh(direction, _p(self.fi), _p(self.u), _p(self.flags), t, flag, _p(p0), _p(p1), _p(p2), _p(bbu))

    def unvoxelize_mesh(self, flag, x0, y0, z0, x1, y1, z1):
        self._cfg()
        self.L.ref_unvoxelize_mesh(_p(self.flags), flag, x0, y0, z0, x1, y1, z1)


class OracleObjective(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("plane_x", ctypes.c_uint32), ("marker", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                ("t_begin", ctypes.c_uint64), ("t_end", ctypes.c_uint64)]


OBJ_KE_PLANE, OBJ_DRAG_X = 1, 2


def objective(kind, t_begin, t_end, plane_x=0, marker=0):
    k = {"ke_plane": OBJ_KE_PLANE, "drag_x": OBJ_DRAG_X}[kind]
    return OracleObjective(k, plane_x, marker, 0, t_begin, t_end)


def _adjoint_lib():
    L = lib()
    if not getattr(L, "_adjoint_typed", False):
        v, d, u64 = ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64
        cfg, obj = ctypes.POINTER(OracleConfig), ctypes.POINTER(OracleObjective)
        L.oracle_objective_f64.argtypes = [cfg, v, v, v, v, v, d, d, d, u64, obj]
        L.oracle_objective_f64.restype = d
        L.oracle_adjoint_f64.argtypes = [cfg, v, v, v, v, v, d, d, d, u64, obj, u64, ctypes.POINTER(d), v]
        L._adjoint_typed = True
    return L


def fp64_objective(o: "Oracle", f0, steps, obj, force=(0.0, 0.0, 0.0), F=None):
    """J of a forward FP64 run of `steps` steps from the initialised DDFs f0 (o must be precision f64)."""
    F = o.F if F is None else np.ascontiguousarray(F, np.float64)
    return float(_adjoint_lib().oracle_objective_f64(ctypes.byref(o.cfg), _p(f0), _p(o.flags), _p(o.rho), _p(o.u), _p(F), *force, steps,
                                                     ctypes.byref(obj)))


def fp64_adjoint(o: "Oracle", f0, steps, obj, interval, force=(0.0, 0.0, 0.0)):
    """(J, dJ/dF) by the checkpointed FP64 discrete adjoint."""
    grad = np.zeros(3 * o.N, np.float64)
    J = ctypes.c_double()
    rc = _adjoint_lib().oracle_adjoint_f64(ctypes.byref(o.cfg), _p(f0), _p(o.flags), _p(o.rho), _p(o.u), _p(o.F), *force, steps,
                                           ctypes.byref(obj), interval, ctypes.byref(J), _p(grad))
    if rc != 0:
        raise RuntimeError("oracle adjoint failed")
    return J.value, grad
