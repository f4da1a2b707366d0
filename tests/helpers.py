"""Shared test helpers: workload generators and comparison metrics."""
from __future__ import annotations

import numpy as np


def rel_err(a, b) -> tuple[float, float]:
    """(max |a-b| / max |b|, ||a-b||_2 / ||b||_2)."""
    a = np.asarray(a, dtype=np.float64); b = np.asarray(b, dtype=np.float64)
    d = a - b
    s = np.abs(b).max() if b.size else 1.0
    n = np.linalg.norm(b) if b.size else 1.0
    return float(np.abs(d).max() / s if d.size else 0.0), float(np.linalg.norm(d) / n if d.size else 0.0)


def stretch_field(X: np.ndarray, seed: int, noise: float = 1e-3, diag=(1.05, 0.98, 0.98)) -> np.ndarray:
    """Affine stretch diag(...) - I applied to X plus i.i.d. N(0, noise^2) nodal noise."""
    rng = np.random.default_rng(seed)
    return ((np.diag(diag) - np.eye(3)) @ X.T).T + noise * rng.standard_normal(X.shape)


def blocks_of(mesh):
    return [(mesh.element_types[b], mesh.element_conns[b]) for b in mesh.element_block_names]
