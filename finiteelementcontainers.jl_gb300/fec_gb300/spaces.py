"""FunctionSpace and the Function types that name the fields
(src/FunctionSpaces.jl, src/Functions.jl)."""
from __future__ import annotations

import numpy as np

from .meshes import ELEMENT_IDS, NNPE, Mesh
from .quadrature import KERNEL_NQ, reference_tables

# quadrature points per element type on the accelerated path (the point counts
# the kernels are built for): 2-point tensor rules for hex8/quad4, 3-point for
# hex27, 1/4 points for tet4/tet10
NUM_QP = dict(KERNEL_NQ)


class FunctionSpace:
    """FunctionSpace(mesh, H1Field, Lagrange): coordinates + block connectivity.

    Connectivity is kept as the reference's flat multi-block Connectivity
    (src/Fields.jl:129-160): `conn_data` concatenates each block's NNPE x NE
    column-major matrix, `conn_offsets` are 1-based block offsets."""

    def __init__(self, mesh: Mesh, field_type: str = "H1Field", interp: str = "Lagrange", *,
                 q_type: str = "GaussLegendre", q_degree: int | None = None):
        if field_type != "H1Field" or interp != "Lagrange":
            raise NotImplementedError("only H1Field/Lagrange spaces are on the assembly path")
        self.q_type, self.q_degree = q_type, q_degree
        self.mesh = mesh
        self.coords = mesh.nodal_coords
        self.block_names = list(mesh.element_block_names)
        self.elem_types = [mesh.element_types[b] for b in self.block_names]
        conns = [mesh.element_conns[b] for b in self.block_names]
        self.block_num_elems = np.array([c.shape[0] for c in conns], dtype=np.int64)
        self.nepes = np.array([NNPE[t] for t in self.elem_types], dtype=np.int64)
        self.conn_data = np.ascontiguousarray(np.concatenate([c.ravel() for c in conns]), dtype=np.int64)
        offs, o = [], 1
        for c in conns:
            offs.append(o)
            o += c.size
        self.conn_offsets = np.array(offs, dtype=np.int64)
        # per block (N, dN, w): the ReferenceFE of each block (src/FunctionSpaces.jl:104-126)
        self.ref_fes = [reference_tables(t, q_type, q_degree) for t in self.elem_types]
        for t, (N, _, _) in zip(self.elem_types, self.ref_fes):
            if N.shape[0] != KERNEL_NQ[t]:
                raise NotImplementedError(f"{t} with {N.shape[0]} quadrature points: the kernels are built for "
                                          f"{KERNEL_NQ[t]}")

    @property
    def num_dimensions(self) -> int:
        return self.coords.shape[1]

    @property
    def num_nodes(self) -> int:
        return self.coords.shape[0]

    def num_blocks(self) -> int:
        return len(self.block_names)

    def num_elements(self, b: int | None = None) -> int:
        return int(self.block_num_elems.sum() if b is None else self.block_num_elems[b - 1])

    def connectivity(self, b: int) -> np.ndarray:
        """Block b's connectivity as (NE, NNPE) (the reference's NNPE x NE view)."""
        o = self.conn_offsets[b - 1] - 1
        n = self.block_num_elems[b - 1] * self.nepes[b - 1]
        return self.conn_data[o:o + n].reshape(-1, self.nepes[b - 1])

    def element_type_ids(self) -> np.ndarray:
        return np.array([ELEMENT_IDS[t] for t in self.elem_types], dtype=np.int32)

    def block_quadrature_sizes(self) -> list[tuple[int, int]]:
        return [(NUM_QP[t], int(n)) for t, n in zip(self.elem_types, self.block_num_elems)]


class ScalarFunction:
    def __init__(self, fspace: FunctionSpace, name: str):
        self.fspace = fspace
        self.names = (name,)


class VectorFunction:
    def __init__(self, fspace: FunctionSpace, name: str):
        self.fspace = fspace
        comps = ("_x", "_y", "_z")[: fspace.num_dimensions]
        self.names = tuple(name + c for c in comps)


def num_fields(var) -> int:
    return len(var.names)
