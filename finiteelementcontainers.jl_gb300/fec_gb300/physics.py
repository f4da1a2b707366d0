"""Physics plugins.

The reference dispatches on AbstractPhysics{NF,NP,NS} subtypes whose
residual/stiffness methods are Julia closures (src/Physics.jl:1-57).  Closures
cannot cross a C ABI, so each physics here is a property block plus an id that
selects a hand-written device implementation; num_fields/num_properties/
num_states mirror the reference's accessors."""
from __future__ import annotations

import numpy as np

from . import _lib


class AbstractPhysics:
    NF = 0
    NP = 0
    NS = 0
    ID = 0

    def num_fields(self) -> int:
        return self.NF

    def num_properties(self) -> int:
        return self.NP

    def num_states(self) -> int:
        return self.NS

    def create_properties(self) -> np.ndarray:
        raise NotImplementedError

    def create_initial_state(self) -> np.ndarray:
        return np.zeros(self.NS, dtype=np.float64)


class Poisson(AbstractPhysics):
    """-div grad u = f with f(X) = amplitude * prod_d sin(pi X_d)
    (test/poisson/TestPoissonCommon.jl:75-107)."""
    NF, NP, NS, ID = 1, 0, 0, _lib.FEC_PHYS_POISSON

    def __init__(self, amplitude: float = 1.0):
        self.amplitude = float(amplitude)

    def create_properties(self):
        return np.array([self.amplitude], dtype=np.float64)


class NeoHookean(AbstractPhysics):
    """Compressible Neo-Hookean solid, psi = K/2 (1/2 (J-1)^2 - ln J) + G/2 (J^{-2/3} tr(F F^T) - 3)
    (test/mechanics/TestMechanicsLargeDeformation.jl:17-27), total Lagrange, 3D."""
    NF, NP, NS, ID = 3, 2, 0, _lib.FEC_PHYS_NEOHOOKEAN

    def __init__(self, bulk_modulus: float, shear_modulus: float):
        self.K = float(bulk_modulus)
        self.G = float(shear_modulus)

    @classmethod
    def from_youngs(cls, E: float, nu: float) -> "NeoHookean":
        return cls(E / (3.0 * (1.0 - 2.0 * nu)), E / (2.0 * (1.0 + nu)))

    def create_properties(self):
        return np.array([self.K, self.G], dtype=np.float64)


class J2Plasticity(AbstractPhysics):
    """Small-strain J2 plasticity with linear isotropic hardening, radial return
    (Simo & Hughes 1998, Box 3.2).  State per point: plastic strain (xx, yy, zz,
    yz, xz, xy) + equivalent plastic strain."""
    NF, NP, NS, ID = 3, 4, 7, _lib.FEC_PHYS_J2

    def __init__(self, E: float, nu: float, yield_stress: float, hardening: float):
        self.E, self.nu, self.sy, self.H = float(E), float(nu), float(yield_stress), float(hardening)

    def create_properties(self):
        return np.array([self.E, self.nu, self.sy, self.H], dtype=np.float64)


def num_fields(p: AbstractPhysics) -> int:
    return p.NF


def num_properties(p: AbstractPhysics) -> int:
    return p.NP


def num_states(p: AbstractPhysics) -> int:
    return p.NS
