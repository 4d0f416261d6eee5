"""Host mirror of the reference's ``class LBM`` (src/lbm.hpp:208-611, src/lbm.cpp:700-1145) over the
C-ABI of include/lbm_capi.h.

Usage follows the reference's setups (src/setup.cpp):

    lbm = LBM(Nx, Ny, Nz, nu, fx, fy, fz, velocity_set=19, collision="trt", storage="fp16s",
              extensions=("equilibrium_boundaries",))
    lbm.flags[n] = TYPE_S; lbm.u.x[n] = 0.05          # host-side set-up
    lbm.run(1000)                                      # copies fields to the GPU, initialises, steps
    lbm.u.read_from_device()                           # brings rho/u up to date and copies them back
    force = lbm.object_force(TYPE_S | TYPE_X)

The reference picks the velocity set, collision operator, DDF storage and extensions with
#defines in src/defines.hpp; here they are constructor keywords with the same meaning.
``arithmetic="exact"`` evaluates the reference's FP32 operation order bit for bit, ``"fast"``
contracts multiply-adds and regroups terms (agreeing to FP32 rounding); the default ``"auto"`` is
exact with FP32 DDF storage and fast with FP16S/FP16C storage.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi as C
from . import vtk as _vtk
from .units import units
from .setups import TYPE_S, TYPE_E, TYPE_T, TYPE_F, TYPE_I, TYPE_G, TYPE_X, TYPE_Y  # noqa: F401


class Field:
    """Host buffer of one device field (the reference's Memory_Container, src/lbm.hpp:239-408).

    ``data`` is the numpy array in the reference layout; ``x``/``y``/``z`` are SoA component views
    for 3-component fields; indexing the Field indexes ``data``.
    """

    NAMES = {C.FIELD_RHO: "rho", C.FIELD_U: "u", C.FIELD_FLAGS: "flags", C.FIELD_F: "F"}

    def __init__(self, lbm: "LBM", field_id: int, dims: int, dtype, fill):
        self.lbm, self.field_id, self.dims = lbm, field_id, dims
        self.name = self.NAMES.get(field_id, "")
        self.data = np.full(lbm.get_N() * dims, fill, dtype=dtype)
        N = lbm.get_N()
        if dims == 3:
            self.x, self.y, self.z = self.data[:N], self.data[N:2 * N], self.data[2 * N:]

    def __getitem__(self, i):
        return self.data[i]

    def __setitem__(self, i, v):
        self.data[i] = v

    def __len__(self):
        return self.data.size

    def length(self):
        return self.lbm.get_N()

    def dimensions(self):
        return self.dims

    def reset(self, value=0):
        self.data[:] = value

    def read_from_device(self):
        """Copies the device field to the host; rho/u are first brought up to date (update_fields)."""
        self.lbm._check(C.load().lbm_read_field(self.lbm._d, self.field_id, self.data.ctypes.data, self.data.nbytes))

    def write_to_device(self):
        self.lbm._check(C.load().lbm_write_field(self.lbm._d, self.field_id, self.data.ctypes.data, self.data.nbytes))

    # ------------------------------------------------------------------ VTK export (src/lbm.hpp:298-340, 401-407)
    def _vtk_units(self, convert_to_si_units):
        if not convert_to_si_units:
            return 1.0, 1.0
        scale = {"rho": units.si_rho(1.0), "u": units.si_u(1.0), "F": units.si_F(1.0)}.get(self.name, 1.0)
        return float(units.si_x(1.0)), float(scale)

    def write_host_to_vtk(self, path="", convert_to_si_units=True):
        """Writes the host copy as <path><name>-<t>.vtk (binary legacy VTK, the reference's format);
        returns the file name. With convert_to_si_units, values and spacing go through ``units``."""
        spacing, scale = self._vtk_units(convert_to_si_units)
        fn = _vtk.default_filename(path, self.name, ".vtk", self.lbm.get_t())
        return _vtk.write_field_vtk(fn, self.data, (self.lbm.get_Nx(), self.lbm.get_Ny(), self.lbm.get_Nz()), self.dims, spacing, scale)

    def write_device_to_vtk(self, path="", convert_to_si_units=True):
        """The same file straight from the device field: the GPU scales, interleaves and byte-swaps
        the values chunk by chunk while the previous chunk is written (lbm_write_vtk); the host copy
        is left as it is."""
        spacing, scale = self._vtk_units(convert_to_si_units)
        fn = _vtk.create_file_extension(_vtk.default_filename(path, self.name, ".vtk", self.lbm.get_t()), ".vtk")
        self.lbm._check(C.load().lbm_write_vtk(self.lbm._d, self.field_id, fn.encode(), spacing, scale))
        return fn


def _ext_bits(extensions) -> int:
    bits = 0
    for e in extensions:
        if e not in C.EXTENSIONS:
            raise ValueError(f"unknown extension {e!r}; known: {sorted(C.EXTENSIONS)}")
        bits |= C.EXTENSIONS[e]
    return bits


class LBM:
    """One LBM domain on one GPU with the reference's LBM interface."""

    def __init__(self, Nx, Ny, Nz, nu, fx=0.0, fy=0.0, fz=0.0, *, velocity_set=19, collision="srt", storage="fp32",
                 extensions=(), device=-1, arithmetic="auto"):
        self.config = C.LBMConfig(int(Nx), int(Ny), int(Nz), int(velocity_set), C.COLLISIONS[collision], C.STORAGES[storage],
                                  _ext_bits(extensions), int(device), float(nu), float(fx), float(fy), float(fz),
                                  C.ARITHMETICS[arithmetic])
        self.arithmetic = arithmetic
        self.velocity_set, self.collision, self.storage = int(velocity_set), collision, storage
        self.extensions = tuple(extensions)
        L = C.load()
        d = ctypes.c_void_p()
        C.check(L.lbm_domain_create(ctypes.byref(self.config), ctypes.byref(d)))
        self._d = d
        self.initialized = False
        self.rho = Field(self, C.FIELD_RHO, 1, np.float32, 1.0)
        self.u = Field(self, C.FIELD_U, 3, np.float32, 0.0)
        self.flags = Field(self, C.FIELD_FLAGS, 1, np.uint8, 0)
        self._F = None

    @property
    def F(self):
        """Host buffer of the force field (allocated on first use: 12 bytes per cell)."""
        if self._F is None:
            self._F = Field(self, C.FIELD_F, 3, np.float32, 0.0)
        return self._F

    # ------------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_d", None):
            C.load().lbm_domain_destroy(self._d)
            self._d = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, status):
        C.check(status)

    @property
    def handle(self):
        return self._d

    # ------------------------------------------------------------------ simulation (src/lbm.cpp:881-984)
    def has_force_field(self) -> bool:
        return bool(self.config.extensions & C.EXT_FORCE_FIELD)

    def initialize(self):
        """Writes rho/u/flags (and F with FORCE_FIELD) to the GPU and runs the initialize kernel."""
        self.rho.write_to_device()
        self.u.write_to_device()
        self.flags.write_to_device()
        if self.has_force_field():
            self.F.write_to_device()
        self._check(C.load().lbm_initialize(self._d))
        self.initialized = True

    def run(self, steps=1, total_steps=None):
        if not self.initialized:
            self.initialize()
        self._check(C.load().lbm_stream_collide(self._d, int(steps)))

    def update_fields(self):
        self._check(C.load().lbm_update_fields(self._d))

    def reset(self):
        self._check(C.load().lbm_reset(self._d))
        self.initialized = False

    def synchronize(self):
        self._check(C.load().lbm_synchronize(self._d))

    # ------------------------------------------------------------------ forces (src/lbm.cpp:991-1015)
    def update_force_field(self):
        self._check(C.load().lbm_update_force_field(self._d))

    def reset_force_field(self):
        self._check(C.load().lbm_reset_force_field(self._d))

    # ------------------------------------------------------------------ moving boundaries (src/lbm.cpp:1019-1023)
    def update_moving_boundaries(self):
        """Marks the cells next to TYPE_S cells with u != 0 as TYPE_MS (and unmarks the others) after
        the solids' velocities changed; needs the "moving_boundaries" extension. Host copies of the
        flags follow before initialization, as after voxelization."""
        self._check(C.load().lbm_update_moving_boundaries(self._d))
        if not self.initialized:
            self.flags.read_from_device()

    def object_center_of_mass(self, flag_marker=TYPE_S):
        out = (ctypes.c_double * 4)()
        self._check(C.load().lbm_object_center_of_mass(self._d, flag_marker, out))
        return np.array(out[:3]), int(out[3])

    def object_force(self, flag_marker=TYPE_S):
        out = (ctypes.c_double * 3)()
        self._check(C.load().lbm_object_force(self._d, flag_marker, out))
        return np.array(out[:3])

    def object_torque(self, rotation_center, flag_marker=TYPE_S):
        out = (ctypes.c_double * 3)()
        cx, cy, cz = (float(v) for v in rotation_center)
        self._check(C.load().lbm_object_torque(self._d, flag_marker, cx, cy, cz, out))
        return np.array(out[:3])

    # ------------------------------------------------------------------ adjoint (new; no reference counterpart)
    def run_adjoint(self, steps, objective="ke_plane", window=None, plane_x=0, marker=TYPE_S, checkpoint_interval=100,
                    workspace_limit_kib=0):
        """Runs `steps` forward time steps (like run) and the checkpointed discrete adjoint back through
        them. Returns (J, dJ/dF, stats): J the objective averaged over the states after the time steps
        of `window` (inclusive, absolute), dJ/dF as a 3N SoA float32 array. F (the per-cell force field,
        FORCE_FIELD) is the design variable; the domain ends at the forward state, t advanced by steps.
        workspace_limit_kib caps the device memory of the adjoint's workspace (0: what is free)."""
        if not self.initialized:
            self.initialize()
        t0 = self.get_t()
        if window is None:
            window = (t0 + steps, t0 + steps)
        cfg = C.AdjointConfig(int(steps), int(checkpoint_interval), C.OBJECTIVES[objective], int(plane_x), int(marker),
                              int(workspace_limit_kib), int(window[0]), int(window[1]))
        J = ctypes.c_double()
        grad = np.empty(3 * self.get_N(), np.float32)
        st = C.AdjointStats()
        self._check(C.load().lbm_run_adjoint(self._d, ctypes.byref(cfg), ctypes.byref(J), grad.ctypes.data, ctypes.byref(st)))
        stats = {k: getattr(st, k) for k, _ in C.AdjointStats._fields_}
        return J.value, grad, stats

    # ------------------------------------------------------------------ geometry (src/lbm.cpp:1074-1093)
    def voxelize_mesh_on_device(self, mesh, flag=TYPE_S, rotation_center=(0.0, 0.0, 0.0), linear_velocity=(0.0, 0.0, 0.0),
                                rotational_velocity=(0.0, 0.0, 0.0)):
        p0 = np.ascontiguousarray(mesh.p0, np.float32)
        p1 = np.ascontiguousarray(mesh.p1, np.float32)
        p2 = np.ascontiguousarray(mesh.p2, np.float32)
        c = (ctypes.c_float * 3)(*rotation_center)
        lv = (ctypes.c_float * 3)(*linear_velocity)
        rv = (ctypes.c_float * 3)(*rotational_velocity)
        self._check(C.load().lbm_voxelize_mesh(self._d, p0.ctypes.data, p1.ctypes.data, p2.ctypes.data, p0.shape[0], flag, c, lv, rv))
        if not self.initialized:  # host copies follow the device, so host-side set-up can continue
            self.flags.read_from_device()
            self.u.read_from_device()

    def write_mesh_to_vtk(self, mesh, path="", convert_to_si_units=True):
        """src/lbm.cpp:1094-1129: the mesh as <path>mesh-<t>.vtk, centred on the box (POLYDATA)."""
        spacing = float(units.si_x(1.0)) if convert_to_si_units else 1.0
        fn = _vtk.default_filename(path, "mesh", ".vtk", self.get_t())
        return _vtk.write_mesh_vtk(fn, mesh, self.center(), spacing)

    def unvoxelize_mesh_on_device(self, mesh, flag=TYPE_S):
        lo = (ctypes.c_float * 3)(*np.asarray(mesh.pmin, np.float32))
        hi = (ctypes.c_float * 3)(*np.asarray(mesh.pmax, np.float32))
        self._check(C.load().lbm_unvoxelize_mesh(self._d, lo, hi, flag))

    # ------------------------------------------------------------------ getters (src/lbm.hpp:448-473)
    def get_Nx(self):
        return self.config.Nx

    def get_Ny(self):
        return self.config.Ny

    def get_Nz(self):
        return self.config.Nz

    def get_N(self):
        return self.config.Nx * self.config.Ny * self.config.Nz

    def get_nu(self):
        return self.config.nu

    def get_tau(self):
        return float(np.float32(3.0) * np.float32(self.config.nu) + np.float32(0.5))

    def get_w(self):
        """Relaxation rate the kernels use."""
        return C.relaxation_rate(self.config.nu)

    def get_t(self):
        t = ctypes.c_uint64()
        self._check(C.load().lbm_get_time_step(self._d, ctypes.byref(t)))
        return t.value

    def get_velocity_set(self):
        return self.velocity_set

    def get_fx(self):
        return self.config.fx

    def get_fy(self):
        return self.config.fy

    def get_fz(self):
        return self.config.fz

    def set_f(self, fx, fy, fz):
        self._check(C.load().lbm_set_force(self._d, fx, fy, fz))
        self.config.fx, self.config.fy, self.config.fz = fx, fy, fz

    def bandwidth_bytes_per_cell(self):
        return int(C.load().lbm_bandwidth_bytes_per_cell(ctypes.byref(self.config)))

    def bytes_per_cell_device(self):
        return int(C.load().lbm_bytes_per_cell_device(ctypes.byref(self.config)))

    # ------------------------------------------------------------------ coordinates (src/lbm.hpp:478-535)
    def coordinates(self, n):
        Nx, Ny = self.config.Nx, self.config.Ny
        t = n % (Nx * Ny)
        return t % Nx, t // Nx, n // (Nx * Ny)

    def index(self, x, y, z):
        return x + (y + z * self.config.Ny) * self.config.Nx

    def position(self, x, y, z):
        return (np.float32(x) - np.float32(0.5) * np.float32(self.config.Nx) + np.float32(0.5),
                np.float32(y) - np.float32(0.5) * np.float32(self.config.Ny) + np.float32(0.5),
                np.float32(z) - np.float32(0.5) * np.float32(self.config.Nz) + np.float32(0.5))

    def size(self):
        return np.array([self.config.Nx, self.config.Ny, self.config.Nz], np.float32)

    def center(self):
        return np.array([0.5 * self.config.Nx - 0.5, 0.5 * self.config.Ny - 0.5, 0.5 * self.config.Nz - 0.5], np.float32)

    # ------------------------------------------------------------------ raw device access
    def device_pointer(self, field_id):
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._check(C.load().lbm_field_device_pointer(self._d, field_id, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def stream(self):
        s = ctypes.c_void_p()
        self._check(C.load().lbm_get_stream(self._d, ctypes.byref(s)))
        return s.value

    def read_ddfs(self):
        """Raw DDF array (q*N, storage dtype) at the current time step."""
        dtype = np.float32 if self.storage == "fp32" else np.uint16
        out = np.empty(self.velocity_set * self.get_N(), dtype=dtype)
        self._check(C.load().lbm_read_field(self._d, C.FIELD_FI, out.ctypes.data, out.nbytes))
        return out
