"""DofManager (src/DofManagers.jl): DOF numbering and Dirichlet elimination."""
from __future__ import annotations

import numpy as np

DIRICHLET_DOF = -1


class DofManager:
    """Global dof = NF*(node-1) + d (1-based).  unknown_dofs is the sorted
    complement of the Dirichlet dofs; dof_to_unknown holds each dof's 1-based
    unknown index or -1 (src/DofManagers.jl:21-73, 227-298)."""

    def __init__(self, var, use_condensed: bool = False):
        if use_condensed:
            raise NotImplementedError("condensed mode is not on the accelerated path")
        self.var = var
        self.nf = len(var.names)
        self.nn = var.fspace.num_nodes
        n = self.nf * self.nn
        self.dirichlet_dofs = np.zeros(0, dtype=np.int64)
        self.unknown_dofs = np.arange(1, n + 1, dtype=np.int64)
        self.dof_to_unknown = np.arange(1, n + 1, dtype=np.int64)

    def __len__(self) -> int:
        return self.nf * self.nn

    @property
    def shape(self) -> tuple[int, int]:
        return (self.nf, self.nn)

    def size(self, i: int | None = None):
        return self.shape if i is None else self.shape[i - 1]

    def function_space(self):
        return self.var.fspace

    def dof_index(self, var_name: str) -> int:
        """0-based field index of a component name (_dof_index_from_var_name)."""
        return self.var.names.index(var_name)


def update_dofs(dof: DofManager, dirichlet_dofs) -> None:
    """update_dofs!(dof, dirichlet_dofs, [], []) (src/DofManagers.jl:227-298)."""
    d = np.unique(np.asarray(dirichlet_dofs, dtype=np.int64))
    n = len(dof)
    if d.size and (d[0] < 1 or d[-1] > n):
        raise IndexError("Dirichlet dof out of range")
    mask = np.ones(n, dtype=bool)
    mask[d - 1] = False
    dof.dirichlet_dofs = d
    dof.unknown_dofs = np.nonzero(mask)[0].astype(np.int64) + 1
    dtu = np.full(n, DIRICHLET_DOF, dtype=np.int64)
    dtu[dof.unknown_dofs - 1] = np.arange(1, dof.unknown_dofs.size + 1, dtype=np.int64)
    dof.dof_to_unknown = dtu


def create_unknowns(dof: DofManager, device=None):
    import torch
    return torch.zeros(dof.unknown_dofs.size, dtype=torch.float64, device=device)


def create_field(dof: DofManager, device=None):
    import torch
    return torch.zeros(len(dof), dtype=torch.float64, device=device)
