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


from fec_gb300.workloads import stretch_field  # noqa: F401  (re-exported for the tests)


def blocks_of(mesh):
    return [(mesh.element_types[b], mesh.element_conns[b]) for b in mesh.element_block_names]
