"""Meshes: the structured box meshes of src/meshes/StructuredMesh.jl and a
block-structured unstructured mesh built from arrays.

Layouts follow the reference: coordinates are dim x NN (stored here as an
(NN, dim) C-order array, which is the same interleaved memory), connectivity
per block is NNPE x NE column-major (stored as (NE, NNPE) C-order), 1-based.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

ELEMENT_IDS = {"HEX8": 1, "QUAD4": 2, "TETRA4": 6, "TETRA10": 7, "HEX27": 8}
NNPE = {"HEX8": 8, "QUAD4": 4, "TETRA4": 4, "TETRA10": 10, "HEX27": 27}
DIM = {"HEX8": 3, "QUAD4": 2, "TETRA4": 3, "TETRA10": 3, "HEX27": 3}
_ALIASES = {"HEX": "HEX8", "QUAD": "QUAD4", "TET": "TETRA4", "TET4": "TETRA4", "TETRA": "TETRA4",
            "TET10": "TETRA10"}


def canonical_element(name: str) -> str:
    n = name.upper()
    n = _ALIASES.get(n, n)
    if n not in ELEMENT_IDS:
        raise ArgumentError(f"Unsupported element type {name}")
    return n


class ArgumentError(ValueError):
    """Mirrors Julia's ArgumentError raised by StructuredMesh for a bad element type."""


def linrange(a: float, b: float, n: int) -> np.ndarray:
    """Julia's LinRange(a, b, n) evaluated element-wise as (1-t)*a + t*b, t=(k-1)/(n-1)."""
    if n == 1:
        return np.array([a], dtype=np.float64)
    t = np.arange(n, dtype=np.float64) / np.float64(n - 1)
    return (1.0 - t) * np.float64(a) + t * np.float64(b)


@dataclass
class Mesh:
    """A mesh with element blocks (the fields of StructuredMesh/UnstructuredMesh
    that the assembly path reads)."""

    nodal_coords: np.ndarray                      # (NN, dim) float64
    element_block_names: list[str]
    element_types: dict[str, str]                 # block name -> canonical element name
    element_conns: dict[str, np.ndarray]          # block name -> (NE, NNPE) int64, 1-based
    nodeset_nodes: dict[str, np.ndarray] = field(default_factory=dict)
    sideset_nodes: dict[str, np.ndarray] = field(default_factory=dict)

    @property
    def num_dimensions(self) -> int:
        return self.nodal_coords.shape[1]

    @property
    def num_nodes(self) -> int:
        return self.nodal_coords.shape[0]

    def num_elements(self) -> int:
        return sum(c.shape[0] for c in self.element_conns.values())


def StructuredMesh(element_type: str, mins, maxs, counts) -> Mesh:
    """StructuredMesh(element_type, mins, maxs, counts) of src/meshes/StructuredMesh.jl:28-83.

    counts are node counts per direction (elements = counts - 1)."""
    if not (len(mins) == len(maxs) == len(counts)):
        raise ValueError("mins, maxs and counts must have the same length")
    for m1, m2 in zip(mins, maxs):
        if m1 >= m2:
            raise IndexError("Dimension has negative or zero length")  # the reference throws BoundsError
    et = element_type.upper()
    # the reference tests occursin(element_type, "HEX"): the name must be a substring of "HEX"
    if et in "HEX":
        coords, conns, nsets = _hex8(mins, maxs, counts)
        etype = "HEX8"
    elif et in "QUAD":
        coords, conns, nsets = _quad4(mins, maxs, counts)
        etype = "QUAD4"
    else:
        raise ArgumentError(f"Unsupported element type {element_type}")
    return Mesh(coords, ["block_1"], {"block_1": etype}, {"block_1": conns}, nsets, dict(nsets))


def _hex8(mins, maxs, counts):
    # src/meshes/StructuredMesh.jl:85-131 and _three_dimensional_coords! (:433-449):
    # coordinate loop nz (bound counts[1]) outer, ny, nx (bound counts[3]) inner
    Nx, Ny, Nz = (int(c) for c in counts)
    xs, ys, zs = linrange(mins[0], maxs[0], Nx), linrange(mins[1], maxs[1], Ny), linrange(mins[2], maxs[2], Nz)
    nz, ny, nx = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    coords = np.stack([xs[nx.ravel()], ys[ny.ravel()], zs[nz.ravel()]], axis=1)

    def node(i, j, k):  # 1-based
        return i + Nx * (j - 1) + Nx * Ny * (k - 1)

    # element loop ex outer, ey, ez inner
    ex, ey, ez = np.meshgrid(np.arange(1, Nx), np.arange(1, Ny), np.arange(1, Nz), indexing="ij")
    ex, ey, ez = ex.ravel(), ey.ravel(), ez.ravel()
    conns = np.stack([node(ex, ey, ez), node(ex + 1, ey, ez), node(ex + 1, ey + 1, ez), node(ex, ey + 1, ez),
                      node(ex, ey, ez + 1), node(ex + 1, ey, ez + 1), node(ex + 1, ey + 1, ez + 1),
                      node(ex, ey + 1, ez + 1)], axis=1).astype(np.int64)
    # _three_dimensional_nsets (:452-470): comprehension, first index fastest
    I = lambda a, b: np.meshgrid(np.arange(1, a + 1), np.arange(1, b + 1), indexing="xy")  # noqa: E731
    i, k = I(Nx, Nz)
    bottom = node(i, 1, k).ravel()
    j, k2 = I(Ny, Nz)
    right = node(Nx, j, k2).ravel()
    i2, j2 = I(Nx, Ny)
    front = node(i2, j2, Nz).ravel()
    top = node(i, Ny, k).ravel()
    left = node(1, j, k2).ravel()
    back = node(i2, j2, 1).ravel()
    nsets = {n: v.astype(np.int64) for n, v in
             dict(bottom=bottom, right=right, front=front, top=top, left=left, back=back).items()}
    return coords, conns, nsets


def _quad4(mins, maxs, counts):
    # src/meshes/StructuredMesh.jl:233-250 and _two_dimensional_coords!
    Nx, Ny = (int(c) for c in counts)
    xs, ys = linrange(mins[0], maxs[0], Nx), linrange(mins[1], maxs[1], Ny)
    ny, nx = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    coords = np.stack([xs[nx.ravel()], ys[ny.ravel()]], axis=1)

    def node(i, j):
        return i + (j - 1) * Nx

    ex, ey = np.meshgrid(np.arange(1, Nx), np.arange(1, Ny), indexing="ij")
    ex, ey = ex.ravel(), ey.ravel()
    conns = np.stack([node(ex, ey), node(ex + 1, ey), node(ex + 1, ey + 1), node(ex, ey + 1)], axis=1)
    nsets = dict(bottom=node(np.arange(1, Nx + 1), 1), right=node(Nx, np.arange(1, Ny + 1)),
                 top=node(np.arange(1, Nx + 1), Ny), left=node(1, np.arange(1, Ny + 1)))
    return coords, conns.astype(np.int64), {k: np.asarray(v, dtype=np.int64) for k, v in nsets.items()}


def UnstructuredMesh(coords, blocks: dict[str, tuple[str, np.ndarray]], nodesets=None, sidesets=None) -> Mesh:
    """A mesh from arrays: coords (NN, dim); blocks name -> (element type, (NE, NNPE) 1-based conn)."""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    names = list(blocks)
    types = {n: canonical_element(blocks[n][0]) for n in names}
    conns = {n: np.ascontiguousarray(blocks[n][1], dtype=np.int64) for n in names}
    for n in names:
        if conns[n].ndim != 2 or conns[n].shape[1] != NNPE[types[n]]:
            raise ValueError(f"block {n}: connectivity must be (NE, {NNPE[types[n]]})")
        if DIM[types[n]] != coords.shape[1]:
            raise ValueError(f"block {n}: {types[n]} is not {coords.shape[1]}D")
    ns = {k: np.asarray(v, dtype=np.int64) for k, v in (nodesets or {}).items()}
    ss = {k: np.asarray(v, dtype=np.int64) for k, v in (sidesets or {}).items()}
    return Mesh(coords, names, types, conns, ns, ss)


# ---------------------------------------------------------------------------
# Box meshes of the element types the reference cannot generate structurally
# (StructuredMesh asserts for tets; it has no hex27).  Used for the mixed
# tet4/tet10/hex27 workloads.
# ---------------------------------------------------------------------------

# Kuhn (Freudenthal) split of a hex into 6 tets around the diagonal 0-6; it is
# conforming across neighbouring hexes of a structured grid.
_KUHN = np.array([[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6], [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]])
# exodus TETRA10 edge order: 4:(0,1) 5:(1,2) 6:(0,2) 7:(0,3) 8:(1,3) 9:(2,3)
TET10_EDGES = np.array([[0, 1], [1, 2], [0, 2], [0, 3], [1, 3], [2, 3]])


def _orient_tets(coords: np.ndarray, tets: np.ndarray) -> np.ndarray:
    x = coords[tets - 1]
    d = np.einsum("ij,ij->i", np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0]), x[:, 3] - x[:, 0])
    neg = d < 0
    tets = tets.copy()
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    return tets


def box_tet4(counts, mins=(0.0, 0.0, 0.0), maxs=(1.0, 1.0, 1.0)) -> Mesh:
    """Box of (counts-1)^3 hexes, each split into 6 positively oriented tet4."""
    hexm = StructuredMesh("hex", mins, maxs, counts)
    h = hexm.element_conns["block_1"]
    tets = h[:, _KUHN].reshape(-1, 4)
    tets = _orient_tets(hexm.nodal_coords, tets)
    return Mesh(hexm.nodal_coords, ["block_1"], {"block_1": "TETRA4"}, {"block_1": tets},
                dict(hexm.nodeset_nodes), {})


def tet4_to_tet10(coords: np.ndarray, tets: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Adds a mid-edge node per unique edge; returns (coords, (NE, 10) conn)."""
    e = tets[:, TET10_EDGES]                        # (NE, 6, 2)
    key = np.sort(e, axis=2).reshape(-1, 2)
    uniq, inv = np.unique(key, axis=0, return_inverse=True)
    mid = 0.5 * (coords[uniq[:, 0] - 1] + coords[uniq[:, 1] - 1])
    new_ids = coords.shape[0] + 1 + inv.reshape(-1, 6)
    return np.concatenate([coords, mid]), np.concatenate([tets, new_ids], axis=1).astype(np.int64)


def box_tet10(counts, mins=(0.0, 0.0, 0.0), maxs=(1.0, 1.0, 1.0)) -> Mesh:
    t4 = box_tet4(counts, mins, maxs)
    coords, conn = tet4_to_tet10(t4.nodal_coords, t4.element_conns["block_1"])
    return Mesh(coords, ["block_1"], {"block_1": "TETRA10"}, {"block_1": conn}, {}, {})


def box_hex27(counts, mins=(0.0, 0.0, 0.0), maxs=(1.0, 1.0, 1.0)) -> Mesh:
    """Box of (counts-1)^3 triquadratic hexes on a (2(counts-1)+1)^3 node grid.
    Local node (i, j, k) in {0,1,2}^3 (coordinates -1, 0, 1) has index i + 3j + 9k."""
    ne = [int(c) - 1 for c in counts]
    M = [2 * n + 1 for n in ne]
    xs = [linrange(mins[d], maxs[d], M[d]) for d in range(3)]
    kz, jy, ix = np.meshgrid(np.arange(M[2]), np.arange(M[1]), np.arange(M[0]), indexing="ij")
    coords = np.stack([xs[0][ix.ravel()], xs[1][jy.ravel()], xs[2][kz.ravel()]], axis=1)
    ex, ey, ez = np.meshgrid(np.arange(ne[0]), np.arange(ne[1]), np.arange(ne[2]), indexing="ij")
    ex, ey, ez = ex.ravel(), ey.ravel(), ez.ravel()
    cols = []
    for k in range(3):
        for j in range(3):
            for i in range(3):
                cols.append(1 + (2 * ex + i) + M[0] * (2 * ey + j) + M[0] * M[1] * (2 * ez + k))
    conn = np.stack(cols, axis=1).astype(np.int64)
    return Mesh(coords, ["block_1"], {"block_1": "HEX27"}, {"block_1": conn}, {}, {})


def merge_meshes(meshes: list[Mesh], names: list[str] | None = None, single_block: bool = False) -> Mesh:
    """Disjoint union of meshes (node ids renumbered, mesh i's nodes and elements
    after those of meshes 0..i-1).  One block per mesh, or, with single_block
    and a common element type, one block holding every element -- so one kernel
    launch covers the whole batch."""
    if single_block:
        types_ = {m.element_types[m.element_block_names[0]] for m in meshes}
        if len(types_) != 1 or any(len(m.element_block_names) != 1 for m in meshes):
            raise ValueError("single_block needs single-block meshes of one element type")
        coords, conns, off = [], [], 0
        for m in meshes:
            b = m.element_block_names[0]
            coords.append(m.nodal_coords)
            conns.append(m.element_conns[b] + off)
            off += m.nodal_coords.shape[0]
        name = (names or ["block_1"])[0]
        return Mesh(np.concatenate(coords), [name], {name: types_.pop()}, {name: np.concatenate(conns)}, {}, {})
    coords, types, conns, off = [], {}, {}, 0
    names = names or [f"block_{i + 1}" for i in range(len(meshes))]
    for name, m in zip(names, meshes):
        if len(m.element_block_names) != 1:
            raise ValueError("merge_meshes takes single-block meshes")
        b = m.element_block_names[0]
        coords.append(m.nodal_coords)
        types[name] = m.element_types[b]
        conns[name] = m.element_conns[b] + off
        off += m.nodal_coords.shape[0]
    return Mesh(np.concatenate(coords), list(names), types, conns, {}, {})
