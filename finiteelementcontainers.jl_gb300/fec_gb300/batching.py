"""Batched assembly of many independent meshes in one set of launches, and the
Newton-type iteration captured as a CUDA graph.

A batch is the disjoint union of its meshes with every element in one element
block: the element kernel and the node gather then cover all meshes in one
launch each, however uneven their sizes.  Each mesh's dofs, residual entries and
CSC columns are contiguous in the batch numbering, so per-mesh results are
views (the merged matrix is block diagonal)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .assemblers import CSCMatrix, assemble_residual_and_stiffness, residual, stiffness
from .meshes import Mesh, StructuredMesh, box_hex27, box_tet4, box_tet10, merge_meshes


def lognormal_cube_sides(count: int = 64, lo: int = 8 ** 3, hi: int = 48 ** 3, seed: int = 2) -> list[int]:
    """Cube sides n_i = round(NE_i^(1/3)) for element counts NE_i drawn log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    ne = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    return [max(1, int(round(x ** (1.0 / 3.0)))) for x in ne]


@dataclass
class Batch:
    mesh: Mesh
    node_offsets: np.ndarray     # (count + 1,) first node of each mesh in the batch numbering
    elem_offsets: np.ndarray     # (count + 1,)

    @property
    def count(self) -> int:
        return len(self.node_offsets) - 1


def batch_of(meshes: list[Mesh]) -> Batch:
    nodes = np.cumsum([0] + [m.num_nodes for m in meshes])
    elems = np.cumsum([0] + [m.num_elements() for m in meshes])
    return Batch(merge_meshes(meshes, single_block=True), nodes.astype(np.int64), elems.astype(np.int64))


def box_batch(sides: list[int]) -> Batch:
    """Unit-cube hex8 meshes with the given numbers of elements per side, batched."""
    return batch_of([StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (n + 1,) * 3) for n in sides])


def mixed_mesh(n_tet4_hex: int, n_tet10_hex: int, n_hex27: int) -> Mesh:
    """Disjoint tet4 / tet10 / hex27 blocks (boxes of the given elements per side;
    each tet box holds 6 n^3 tets)."""
    return merge_meshes([box_tet4((n_tet4_hex + 1,) * 3), box_tet10((n_tet10_hex + 1,) * 3),
                         box_hex27((n_hex27 + 1,) * 3)], names=["tet4", "tet10", "hex27"])


def mesh_system(asm, batch: Batch, i: int) -> tuple[object, CSCMatrix]:
    """Residual and CSC tangent of mesh i of a batch assembled without Dirichlet
    dofs (views into the batch results)."""
    nf = asm.dof.nf
    if asm.dof.unknown_dofs.size != len(asm.dof):
        raise ValueError("mesh_system needs a batch without Dirichlet dofs")
    c0, c1 = nf * int(batch.node_offsets[i]), nf * int(batch.node_offsets[i + 1])
    K = stiffness(asm)
    z0, z1 = int(K.colptr[c0]) - 1, int(K.colptr[c1]) - 1
    colptr = K.colptr[c0:c1 + 1] - z0
    rowval = K.rowval[z0:z1] - c0
    return residual(asm)[c0:c1], CSCMatrix(c1 - c0, colptr, rowval, K.nzval[z0:z1])


class NewtonLoop:
    """`iterations` fused residual + tangent assemblies of one or more
    (assembler, parameters, unknowns) systems, each followed by the diagonally
    preconditioned update Uu <- Uu - damping * R / diag(K), recorded once and
    replayed as a single CUDA graph.  The residual norms of every iteration are
    kept on the device (`norms`).  The linear solve of a full Newton step is not
    part of the assembly path; the diagonal update keeps each iteration's input
    dependent on the previous iteration's assembled R and K."""

    def __init__(self, systems, iterations: int = 5, damping: float = 0.5, precision: str | None = None):
        import torch
        self.torch = torch
        self.systems = []
        for asm, p, Uu in systems:
            colptr, rowval = asm.pattern()
            n = colptr.size - 1
            cols = np.repeat(np.arange(n), np.diff(colptr))
            diag = np.nonzero(rowval - 1 == cols)[0]
            if diag.size != n:
                raise ValueError("every unknown needs a diagonal entry")
            self.systems.append((asm, p, Uu.clone(), torch.from_numpy(diag).to(Uu.device)))
        self.iterations = iterations
        self.damping = damping
        self.precision = precision
        self.norms = torch.zeros(len(self.systems), iterations, dtype=torch.float64, device=Uu.device)
        self.graph = None

    def _body(self):
        for it in range(self.iterations):
            for s, (asm, p, Uu, diag) in enumerate(self.systems):
                R, K = assemble_residual_and_stiffness(asm, Uu, p, precision=self.precision)
                Uu.sub_(self.damping * R / K.nzval[diag])
                self.norms[s, it] = R.norm()

    def run_eager(self):
        self._body()

    def capture(self):
        torch = self.torch
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        saved = [Uu.clone() for _, _, Uu, _ in self.systems]
        with torch.cuda.stream(side):  # warm-up outside the graph (allocations, attributes)
            self._body()
        torch.cuda.current_stream().wait_stream(side)
        for (_, _, Uu, _), u0 in zip(self.systems, saved):
            Uu.copy_(u0)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._body()
        return self

    def replay(self):
        self.graph.replay()

    def unknowns(self, s: int = 0):
        return self.systems[s][2]
