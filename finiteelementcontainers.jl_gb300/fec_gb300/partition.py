"""Partitioned assembly: the domain decomposition of ext/PartitionedArraysExt.jl
(per-part serial assembly, then one exchange that adds ghost contributions into
their owners, :313-366, 449-481), built on the single-GPU assembler.

Elements are split into contiguous ranges, one per part.  A part holds the
nodes its elements touch (owned and ghost) under a local numbering, assembles
its local residual and CSC tangent over its local unknowns with the ordinary
kernels, and maps every local entry to its position in the global system
(`unknown_l2g` for the residual, `kmap` for nzval).  The global system is then
one exchange:

  * on one GPU (`PartitionedAssembler`): every part's entries are added into
    zeroed global arrays, part by part in increasing order;
  * across ranks (`exchange_to_owners`): each global column is owned by the
    lowest part touching its node; a part sends the entries of columns it does
    not own to their owners (point-to-point), and each owner adds, into zeroed
    owned columns, its own entries and then what it receives in increasing
    part order.

Both add every entry's part sums in the same order, so they give identical
results; they equal the single-part assembly up to the regrouping of each
entry's element sum by part (<= 1e-12 relative)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .assemblers import SparseMatrixAssembler, assemble_residual_and_stiffness, create_parameters, update_dofs_bcs
from .dofs import DofManager, update_dofs
from .meshes import Mesh, UnstructuredMesh
from .spaces import FunctionSpace, ScalarFunction, VectorFunction


@dataclass
class Part:
    index: int
    elems: tuple[int, int]       # global element range [e0, e1)
    nodes: np.ndarray            # sorted global node ids (1-based) touched by the part
    mesh: Mesh                   # the part's elements over its local node numbering
    dof_to_unknown: np.ndarray   # local dof -> local unknown (1-based) or -1
    unknown_l2g: np.ndarray      # local unknown (0-based) -> global unknown (0-based), increasing
    owner_of_col: np.ndarray     # owning part of each local unknown's column
    kmap: np.ndarray | None = None   # local nz (0-based) -> global nz (0-based), increasing

    @property
    def owned_cols(self) -> np.ndarray:
        return self.owner_of_col == self.index


def element_ranges(num_elems: int, nparts: int) -> list[tuple[int, int]]:
    b = np.linspace(0, num_elems, nparts + 1).round().astype(np.int64)
    return [(int(b[i]), int(b[i + 1])) for i in range(nparts)]


def _var(mesh: Mesh, nf: int):
    V = FunctionSpace(mesh)
    return ScalarFunction(V, "u") if nf == 1 else VectorFunction(V, "u")


def build_parts(mesh: Mesh, nf: int, dof_to_unknown: np.ndarray, nparts: int) -> list[Part]:
    """Partitions of a single-block mesh given the global DOF numbering."""
    if len(mesh.element_block_names) != 1:
        raise ValueError("partitioning takes a single-block mesh")
    bname = mesh.element_block_names[0]
    conn = mesh.element_conns[bname]
    etype = mesh.element_types[bname]
    first_part = np.full(mesh.num_nodes + 1, nparts, dtype=np.int64)
    staged = []
    for p, (e0, e1) in enumerate(element_ranges(conn.shape[0], nparts)):
        c = conn[e0:e1]
        nodes = np.unique(c)
        first_part[nodes] = np.minimum(first_part[nodes], p)
        lmesh = UnstructuredMesh(mesh.nodal_coords[nodes - 1], {bname: (etype, np.searchsorted(nodes, c) + 1)})
        gdofs = (nf * (nodes[:, None] - 1) + np.arange(nf)[None, :]).ravel()     # local dof -> global dof (0-based)
        gdtu = dof_to_unknown[gdofs]
        unknown = gdtu > 0
        ldtu = np.full(gdofs.size, -1, dtype=np.int64)
        ldtu[unknown] = np.arange(1, int(unknown.sum()) + 1)
        staged.append((p, (e0, e1), nodes, lmesh, ldtu, (gdtu[unknown] - 1).astype(np.int64), unknown))
    parts = []
    for p, er, nodes, lmesh, ldtu, l2g, unknown in staged:
        node_of_col = np.repeat(nodes, nf)[unknown]
        parts.append(Part(p, er, nodes, lmesh, ldtu, l2g, first_part[node_of_col]))
    return parts


def local_pattern_map(part: Part, local_colptr: np.ndarray, local_rowval: np.ndarray, colptr: np.ndarray,
                      rowval: np.ndarray) -> np.ndarray:
    """Global nz position of every local CSC entry (all patterns 1-based)."""
    l2g = part.unknown_l2g
    kmap = np.empty(local_rowval.size, dtype=np.int64)
    for c in range(local_colptr.size - 1):
        s, t = local_colptr[c] - 1, local_colptr[c + 1] - 1
        if s == t:
            continue
        G = l2g[c]
        g0, g1 = colptr[G] - 1, colptr[G + 1] - 1
        kmap[s:t] = g0 + np.searchsorted(rowval[g0:g1] - 1, l2g[local_rowval[s:t] - 1])
    if not np.array_equal(rowval[kmap] - 1, l2g[local_rowval - 1]):
        raise RuntimeError("a local entry is missing from the global pattern")
    return kmap


def part_pattern(part: Part, colptr: np.ndarray, rowval: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Local CSC pattern of a part (host-side symbolic phase) and its map into the global pattern."""
    asm = SparseMatrixAssembler(_var(part.mesh, part.dof_to_unknown.size // part.nodes.size), device=-1)
    update_dofs(asm.dof, np.nonzero(part.dof_to_unknown < 0)[0] + 1)
    asm._push_dofs()
    lcp, lrv = asm.pattern()
    part.kmap = local_pattern_map(part, lcp, lrv, colptr, rowval)
    return lcp, lrv


class PartitionedAssembler:
    """N logical parts of one mesh assembled on one GPU, combined by the exchange
    into the global residual over unknowns and the global CSC nzval."""

    def __init__(self, mesh: Mesh, physics, nparts: int, *, dirichlet_bcs=(), device: int = 0,
                 precision: str = "fp64"):
        import torch
        nf = physics.NF
        # global numbering and pattern: the host-side symbolic phase of the whole mesh
        self.host = SparseMatrixAssembler(_var(mesh, nf), device=-1)
        update_dofs_bcs(self.host, list(dirichlet_bcs))
        self.dof: DofManager = self.host.dof
        self.colptr, self.rowval = self.host.pattern()
        self.nnz = int(self.rowval.size)
        self.parts = build_parts(mesh, nf, self.dof.dof_to_unknown, nparts)
        dev = f"cuda:{device}"
        gvals = np.zeros(len(self.dof))   # Dirichlet values, evaluated at t = 0
        for bc in dirichlet_bcs:
            d, nodes = bc.dofs_and_nodes(mesh, self.dof)
            gvals[d - 1] = [bc.func(mesh.nodal_coords[n - 1], 0.0) for n in nodes]
        self.local = []
        for part in self.parts:
            asm, p = local_assembler(part, physics, gvals, self.colptr, self.rowval, device=device,
                                     precision=precision)
            self.local.append((asm, p, torch.from_numpy(part.unknown_l2g).to(dev),
                               torch.from_numpy(part.kmap).to(dev)))
        self.R = torch.zeros(self.dof.unknown_dofs.size, dtype=torch.float64, device=dev)
        self.nzval = torch.zeros(self.nnz, dtype=torch.float64, device=dev)

    def assemble(self, Uu):
        """Global residual and nzval for the global unknowns Uu (a device tensor)."""
        self.R.zero_()
        self.nzval.zero_()
        for asm, p, l2g, kmap in self.local:
            R_l, K_l = assemble_residual_and_stiffness(asm, Uu.index_select(0, l2g), p)
            # the exchange on one GPU: a part's targets are distinct, parts are added in order
            self.R.index_add_(0, l2g, R_l)
            self.nzval.index_add_(0, kmap, K_l.nzval)
        return self.R, self.nzval


def local_assembler(part: Part, physics, dirichlet_values: np.ndarray, colptr: np.ndarray, rowval: np.ndarray, *,
                    device: int = 0, precision: str = "fp64"):
    """A part's own assembler and parameters on `device`: its elements over its
    local numbering, its local unknowns (the global Dirichlet dofs among its
    nodes stay Dirichlet, with their global values), and part.kmap set from its
    pattern.  Its assemblies take the part's unknowns,
    Uu_global[part.unknown_l2g]."""
    import torch
    nf = part.dof_to_unknown.size // part.nodes.size
    asm = SparseMatrixAssembler(_var(part.mesh, nf), device=device, precision=precision)
    p = create_parameters(part.mesh, asm, physics)
    ldd = np.nonzero(part.dof_to_unknown < 0)[0] + 1
    update_dofs(asm.dof, ldd)
    asm._push_dofs()
    gdofs = (nf * (part.nodes[:, None] - 1) + np.arange(nf)[None, :]).ravel()
    dev = f"cuda:{device}"
    p.bc_dofs = torch.as_tensor(ldd, dtype=torch.int64).to(dev)
    p.bc_vals = torch.as_tensor(dirichlet_values[gdofs[ldd - 1]], dtype=torch.float64).to(dev)
    lcp, lrv = asm.pattern()
    part.kmap = local_pattern_map(part, lcp, lrv, colptr, rowval)
    return asm, p


def owned_positions(part: Part, colptr: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Global unknowns and global nz positions of the columns a part owns."""
    cols = part.unknown_l2g[part.owned_cols]
    pos = np.concatenate([np.arange(colptr[G] - 1, colptr[G + 1] - 1) for G in cols]) if cols.size else \
        np.zeros(0, dtype=np.int64)
    return cols, pos.astype(np.int64)


def exchange_to_owners(part: Part, R_local: np.ndarray, nz_local: np.ndarray, rank: int, world: int,
                       colptr: np.ndarray, group=None):
    """The exchange across ranks with torch.distributed point-to-point messages.

    Rank `rank` holds part `rank`'s local residual and nzval.  Returns the global
    unknowns it owns with their residual, and the global nz positions of its
    owned columns with their values."""
    import torch
    import torch.distributed as dist
    l2g, kmap = part.unknown_l2g, part.kmap
    gcol_of_nz = np.searchsorted(colptr - 1, kmap, side="right") - 1
    owner_of_nz = part.owner_of_col[np.searchsorted(l2g, gcol_of_nz)]
    own_cols, own_pos = owned_positions(part, colptr)
    R_own = np.zeros(own_cols.size)
    nz_own = np.zeros(own_pos.size)
    R_own[np.searchsorted(own_cols, l2g[part.owned_cols])] += R_local[part.owned_cols]
    mine = owner_of_nz == rank
    nz_own[np.searchsorted(own_pos, kmap[mine])] += nz_local[mine]
    for dst in range(rank):  # owners of this part's ghost columns have lower ranks
        rm = part.owner_of_col == dst
        km = owner_of_nz == dst
        payload = [torch.from_numpy(l2g[rm]), torch.from_numpy(R_local[rm]), torch.from_numpy(kmap[km]),
                   torch.from_numpy(nz_local[km])]
        dist.send(torch.tensor([t.numel() for t in payload], dtype=torch.int64), dst, group=group)
        for t in payload:
            if t.numel():
                dist.send(t.contiguous(), dst, group=group)
    for src in range(rank + 1, world):  # contributions added in increasing part order
        sizes = torch.zeros(4, dtype=torch.int64)
        dist.recv(sizes, src, group=group)
        bufs = [torch.zeros(int(sizes[0]), dtype=torch.int64), torch.zeros(int(sizes[1]), dtype=torch.float64),
                torch.zeros(int(sizes[2]), dtype=torch.int64), torch.zeros(int(sizes[3]), dtype=torch.float64)]
        for b in bufs:
            if b.numel():
                dist.recv(b, src, group=group)
        np.add.at(R_own, np.searchsorted(own_cols, bufs[0].numpy()), bufs[1].numpy())
        np.add.at(nz_own, np.searchsorted(own_pos, bufs[2].numpy()), bufs[3].numpy())
    return own_cols, R_own, own_pos, nz_own
