"""Dirichlet boundary conditions (src/bcs/DirichletBCs.jl, BoundaryConditions.jl)."""
from __future__ import annotations

import numpy as np


class DirichletBC:
    """DirichletBC(var_name, func; nodeset_name | sideset_name | block_name).

    func(X, t) gives the value at a node with coordinates X."""

    def __init__(self, var_name: str, func, *, block_name=None, nodeset_name=None, sideset_name=None):
        given = [x is not None for x in (block_name, nodeset_name, sideset_name)]
        if sum(given) == 0:
            raise ValueError("block_name, nodeset_name, or sideset_name required as input arguments in DirichletBC")
        if sum(given) != 1:
            raise ValueError("More than one entity type specificed in DirichletBC")
        self.var_name = var_name
        self.func = func
        self.block_name = block_name
        self.nodeset_name = nodeset_name
        self.sideset_name = sideset_name

    def nodes(self, mesh) -> np.ndarray:
        if self.block_name is not None:
            return np.unique(mesh.element_conns[self.block_name])
        if self.nodeset_name is not None:
            return np.asarray(mesh.nodeset_nodes[self.nodeset_name], dtype=np.int64)
        return np.asarray(mesh.sideset_nodes[self.sideset_name], dtype=np.int64)

    def dofs_and_nodes(self, mesh, dof):
        """Sorted unique dofs with their nodes (DirichletBCContainer, DirichletBCs.jl:64-89)."""
        k = dof.dof_index(self.var_name)
        nodes = self.nodes(mesh)
        dofs = dof.nf * (nodes - 1) + k + 1
        u, idx = np.unique(dofs, return_index=True)
        return u.astype(np.int64), nodes[idx]


def dirichlet_dofs(bcs, mesh, dof) -> np.ndarray:
    """unique(sort(all bc dofs)) (DirichletBCs.jl:396-398)."""
    if not bcs:
        return np.zeros(0, dtype=np.int64)
    return np.unique(np.concatenate([bc.dofs_and_nodes(mesh, dof)[0] for bc in bcs]))
