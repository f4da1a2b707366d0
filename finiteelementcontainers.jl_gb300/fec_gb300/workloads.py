"""Seeded synthetic inputs of the benchmark workloads."""
from __future__ import annotations

import numpy as np


def stretch_field(X: np.ndarray, seed: int, noise: float = 1e-3, diag=(1.05, 0.98, 0.98)) -> np.ndarray:
    """Displacement (diag(...) - I) X plus i.i.d. N(0, noise^2) nodal noise, shape of X."""
    rng = np.random.default_rng(seed)
    return ((np.diag(diag) - np.eye(3)) @ X.T).T + noise * rng.standard_normal(X.shape)


def uniaxial_path(X: np.ndarray, step: int, nsteps: int = 20, final_strain: float = 0.01, nu: float = 0.3,
                  noise: float = 1e-5, seed: int = 3) -> np.ndarray:
    """Displacement of load step `step` (1-based) of a monotone uniaxial stretch to
    `final_strain` in `nsteps` steps: (e x, -nu e y, -nu e z) with e = final_strain *
    step / nsteps, plus i.i.d. N(0, noise^2) nodal noise drawn per step."""
    e = final_strain * min(step, nsteps) / nsteps
    rng = np.random.default_rng(seed * 1000 + step)
    U = np.stack([e * X[:, 0], -nu * e * X[:, 1], -nu * e * X[:, 2]], axis=1)
    return U + noise * rng.standard_normal(X.shape)


def uniaxial_bcs():
    """Symmetry on the x-, y-, z- faces and a prescribed x displacement on the x+
    face; the values are set per load step from `uniaxial_path`."""
    from .bcs import DirichletBC

    def zero(X, t):
        return 0.0
    return [DirichletBC("u_x", zero, nodeset_name="left"), DirichletBC("u_y", zero, nodeset_name="bottom"),
            DirichletBC("u_z", zero, nodeset_name="back"), DirichletBC("u_x", zero, nodeset_name="right")]


def uniaxial_inputs(X: np.ndarray, unknown_dofs: np.ndarray, bc_dofs: np.ndarray, nsteps: int = 20,
                    final_strain: float = 0.01) -> list[tuple[np.ndarray, np.ndarray]]:
    """Per load step of `uniaxial_path`: (values at the unknowns, values at the
    Dirichlet dofs), dof numbers 1-based."""
    out = []
    for s in range(1, nsteps + 1):
        U = uniaxial_path(X, s, nsteps=nsteps, final_strain=final_strain).ravel()
        out.append((np.ascontiguousarray(U[unknown_dofs - 1]), np.ascontiguousarray(U[bc_dofs - 1])))
    return out
