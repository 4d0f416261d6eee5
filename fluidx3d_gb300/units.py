"""Unit conversion between lattice and SI units (the reference's ``Units``, src/units.hpp:5-75), used
by the VTK export to write SI values. ``units`` is the module-wide instance, like the reference's
global ``units``; its default is the identity (1 cell = 1 m, 1 time step = 1 s, density 1 = 1 kg/m^3).
All conversions are FP32, in the reference's operation order."""
from __future__ import annotations

import numpy as np

f32 = np.float32


class Units:
    def __init__(self):
        self.unit_m, self.unit_kg, self.unit_s = f32(1.0), f32(1.0), f32(1.0)

    def set_m_kg_s(self, *args):
        """set_m_kg_s(x, u, rho, si_x, si_u, si_rho): a length x, velocity u and density rho in lattice
        units equal si_x [m], si_u [m/s] and si_rho [kg/m^3] (src/units.hpp:9-14);
        set_m_kg_s(m, kg, s): the base units directly (src/units.hpp:15-20)."""
        if len(args) == 6:
            x, u, rho, si_x, si_u, si_rho = (f32(a) for a in args)
            self.unit_m = f32(si_x / x)
            self.unit_kg = f32(f32(si_rho / rho) * f32(f32(self.unit_m * self.unit_m) * self.unit_m))
            self.unit_s = f32(f32(u / si_u) * self.unit_m)
        elif len(args) == 3:
            self.unit_m, self.unit_kg, self.unit_s = (f32(a) for a in args)
        else:
            raise TypeError("set_m_kg_s takes (x, u, rho, si_x, si_u, si_rho) or (m, kg, s)")

    # lattice -> SI (src/units.hpp:58-71)
    def si_x(self, x):
        return f32(f32(x) * self.unit_m)

    def si_t(self, t):
        return f32(f32(t) * self.unit_s)

    def si_u(self, u):
        return f32(f32(f32(u) * self.unit_m) / self.unit_s)

    def si_rho(self, rho):
        return f32(f32(f32(rho) * self.unit_kg) / f32(f32(self.unit_m * self.unit_m) * self.unit_m))

    def si_nu(self, nu):
        return f32(f32(f32(nu) * f32(self.unit_m * self.unit_m)) / self.unit_s)

    def si_F(self, F):
        return f32(f32(f32(f32(F) * self.unit_kg) * self.unit_m) / f32(self.unit_s * self.unit_s))

    # SI -> lattice (src/units.hpp:37-50)
    def x(self, si_x):
        return f32(f32(si_x) / self.unit_m)

    def u(self, si_u):
        return f32(f32(f32(si_u) * self.unit_s) / self.unit_m)

    def rho(self, si_rho):
        return f32(f32(f32(si_rho) * f32(f32(self.unit_m * self.unit_m) * self.unit_m)) / self.unit_kg)

    def nu(self, si_nu):
        return f32(f32(f32(si_nu) * self.unit_s) / f32(self.unit_m * self.unit_m))

    def F(self, si_F):
        return f32(f32(f32(si_F) * f32(self.unit_s * self.unit_s)) / f32(self.unit_kg * self.unit_m))

    def t(self, si_t):  # to_ulong (src/utilities.hpp:514-516): truncation of max(x + 0.5, 0.5)
        return int(max(float(f32(f32(f32(si_t) / self.unit_s) + f32(0.5))), 0.5))


units = Units()
