"""Seeded synthetic inputs of the benchmark workloads."""
from __future__ import annotations

import numpy as np


def stretch_field(X: np.ndarray, seed: int, noise: float = 1e-3, diag=(1.05, 0.98, 0.98)) -> np.ndarray:
    """Displacement (diag(...) - I) X plus i.i.d. N(0, noise^2) nodal noise, shape of X."""
    rng = np.random.default_rng(seed)
    return ((np.diag(diag) - np.eye(3)) @ X.T).T + noise * rng.standard_normal(X.shape)
