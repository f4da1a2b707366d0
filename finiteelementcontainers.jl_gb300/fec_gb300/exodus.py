"""Exodus II mesh and nodal-field I/O (the reference's src/meshes/Exodus.jl and
src/PostProcessors.jl, which read and write through Exodus.jl).

Exodus II files are netCDF classic or 64-bit-offset files with fixed names:
`coordx/coordy/coordz` (or `coord`), one `connect<i>` per element block with an
`elem_type` attribute, block ids in `eb_prop1` and names in `eb_names`, node
sets `node_ns<i>` (ids `ns_prop1`, names `ns_names`), side sets
`elem_ss<i>`/`side_ss<i>`, and the results: `time_whole` over the unlimited
`time_step` dimension, `name_nod_var` and `vals_nod_var<k>`.  The netCDF layer
is scipy's netCDF-3 reader/writer; this module maps it to meshes and fields.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .meshes import ArgumentError, Mesh, UnstructuredMesh, canonical_element

LEN_STRING = 33

# Exodus II side numbering: local nodes (1-based) of side s of an element.
SIDE_NODES = {
    "QUAD4": [[1, 2], [2, 3], [3, 4], [4, 1]],
    "HEX8": [[1, 2, 6, 5], [2, 3, 7, 6], [3, 4, 8, 7], [1, 5, 8, 4], [1, 4, 3, 2], [5, 6, 7, 8]],
    "TETRA4": [[1, 2, 4], [2, 3, 4], [1, 4, 3], [1, 3, 2]],
    "TETRA10": [[1, 2, 4, 5, 9, 8], [2, 3, 4, 6, 10, 9], [1, 4, 3, 8, 10, 7], [1, 3, 2, 7, 6, 5]],
}


def _netcdf():
    from scipy.io import netcdf_file
    return netcdf_file


def _chars(a) -> str:
    """A netCDF char array (bytes) as a str, trailing NULs and blanks removed."""
    b = np.asarray(a).tobytes() if not isinstance(a, (bytes, str)) else a
    if isinstance(b, str):
        return b.strip("\x00 ").strip()
    return b.split(b"\x00")[0].decode(errors="replace").strip()


def _names(v, key: str, n: int, prefix: str, ids) -> list[str]:
    out = []
    if key in v:
        arr = v[key][:]
        for i in range(n):
            out.append(_chars(arr[i]))
    return [nm if nm else f"{prefix}_{int(ids[i])}" for i, nm in enumerate(out or [""] * n)]


class ExodusFile:
    """An Exodus II database opened for reading (FileMesh(ExodusMesh, file),
    src/meshes/Exodus.jl:18-146): element blocks, coordinates, node and side
    sets, id maps and the stored nodal results."""

    def __init__(self, path):
        self.path = str(path)
        self._f = _netcdf()(self.path, "r", mmap=False)
        self._v = self._f.variables
        self._d = self._f.dimensions

    def close(self) -> None:
        self._f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _dim(self, name: str, default: int = 0) -> int:
        d = self._d.get(name, None)
        return default if d is None else int(d)

    def num_dimensions(self) -> int:
        return self._dim("num_dim")

    def num_nodes(self) -> int:
        return self._dim("num_nodes")

    def nodal_coordinates(self) -> np.ndarray:
        """(NN, dim) float64."""
        nd, v = self.num_dimensions(), self._v
        if "coordx" in v:
            cols = [np.asarray(v[c][:], dtype=np.float64) for c in ("coordx", "coordy", "coordz")[:nd]]
            return np.ascontiguousarray(np.stack(cols, axis=1))
        return np.ascontiguousarray(np.asarray(v["coord"][:], dtype=np.float64)[:nd].T)

    def node_id_map(self) -> np.ndarray:
        v = self._v
        if "node_num_map" in v:
            return np.asarray(v["node_num_map"][:], dtype=np.int64)
        return np.arange(1, self.num_nodes() + 1, dtype=np.int64)

    def element_ids(self) -> np.ndarray:
        v = self._v
        if "elem_num_map" in v:
            return np.asarray(v["elem_num_map"][:], dtype=np.int64)
        return np.arange(1, self._dim("num_elem") + 1, dtype=np.int64)

    def element_blocks(self) -> dict[str, tuple[str, np.ndarray]]:
        """Block name -> (Exodus element type, (NE, NNPE) 1-based connectivity)."""
        nb, v = self._dim("num_el_blk"), self._v
        ids = np.asarray(v["eb_prop1"][:], dtype=np.int64) if "eb_prop1" in v else np.arange(1, nb + 1)
        names = _names(v, "eb_names", nb, "block", ids)
        out = {}
        for i in range(nb):
            c = v[f"connect{i + 1}"]
            et = c.elem_type
            out[names[i]] = (_chars(et), np.asarray(c[:], dtype=np.int64).reshape(c.shape))
        return out

    def nodesets(self) -> dict[str, np.ndarray]:
        n, v = self._dim("num_node_sets"), self._v
        if n == 0:
            return {}
        ids = np.asarray(v["ns_prop1"][:], dtype=np.int64) if "ns_prop1" in v else np.arange(1, n + 1)
        names = _names(v, "ns_names", n, "nset", ids)
        return {names[i]: np.asarray(v[f"node_ns{i + 1}"][:], dtype=np.int64) for i in range(n)}

    def sidesets(self) -> dict[str, tuple[np.ndarray, np.ndarray]]:
        """Side set name -> (elements, sides), both 1-based."""
        n, v = self._dim("num_side_sets"), self._v
        if n == 0:
            return {}
        ids = np.asarray(v["ss_prop1"][:], dtype=np.int64) if "ss_prop1" in v else np.arange(1, n + 1)
        names = _names(v, "ss_names", n, "sset", ids)
        return {names[i]: (np.asarray(v[f"elem_ss{i + 1}"][:], dtype=np.int64),
                           np.asarray(v[f"side_ss{i + 1}"][:], dtype=np.int64)) for i in range(n)}

    def times(self) -> np.ndarray:
        v = self._v
        return np.asarray(v["time_whole"][:], dtype=np.float64) if "time_whole" in v else np.zeros(0)

    def nodal_variable_names(self) -> list[str]:
        v = self._v
        if "name_nod_var" not in v:
            return []
        arr = v["name_nod_var"][:]
        return [_chars(arr[i]) for i in range(arr.shape[0])]

    def nodal_variable(self, name: str, time_index: int) -> np.ndarray:
        """Values of nodal variable `name` at 1-based time_index."""
        k = self.nodal_variable_names().index(name) + 1
        return np.asarray(self._v[f"vals_nod_var{k}"][time_index - 1], dtype=np.float64).copy()


def _element_of_blocks(blocks, elem_global: np.ndarray):
    """(block name, local element 0-based) of each global 1-based element id."""
    names = list(blocks)
    starts = np.cumsum([0] + [blocks[n][1].shape[0] for n in names])
    b = np.searchsorted(starts, elem_global - 1, side="right") - 1
    return [names[i] for i in b], elem_global - 1 - starts[b]


def sideset_nodes(blocks, elems: np.ndarray, sides: np.ndarray) -> np.ndarray:
    """Sorted unique 1-based nodes on the given element sides."""
    names, local = _element_of_blocks(blocks, elems)
    nodes = []
    for name, e, s in zip(names, local, sides):
        et, conn = blocks[name]
        table = SIDE_NODES.get(canonical_element(et))
        if table is None:
            raise NotImplementedError(f"side sets of {et} elements")
        nodes.extend(conn[e][np.asarray(table[int(s) - 1]) - 1])
    return np.unique(np.asarray(nodes, dtype=np.int64))


def read_exodus(path) -> Mesh:
    """UnstructuredMesh(mesh_file) of an Exodus II file (src/meshes/UnstructuredMesh.jl):
    coordinates, element blocks, node sets, and side sets as their nodes."""
    with ExodusFile(path) as f:
        coords = f.nodal_coordinates()
        raw = f.element_blocks()
        for name, (et, _) in raw.items():
            try:
                canonical_element(et)
            except ArgumentError as ex:
                raise ArgumentError(f"{Path(str(path)).name}: block {name}: {ex}") from None
        ns = f.nodesets()
        ss = {name: sideset_nodes(raw, el, sd) for name, (el, sd) in f.sidesets().items()}
    return UnstructuredMesh(coords, raw, nodesets=ns, sidesets=ss)


def _put_names(f, var: str, dim: str, names: list[str]) -> None:
    v = f.createVariable(var, "c", (dim, "len_string"))
    arr = np.zeros((len(names), LEN_STRING), dtype="S1")
    for i, nm in enumerate(names):
        b = nm.encode()[:LEN_STRING - 1]
        arr[i, :len(b)] = np.frombuffer(b, dtype="S1")
    v[:] = arr


class ExodusPostProcessor:
    """PostProcessor(mesh, output_file, vars...) with write_times / write_field
    (src/PostProcessors.jl:15-82, src/meshes/Exodus.jl:148-282): writes the mesh
    and declares the nodal variables once, then stores one value per node and
    time step.  The file is complete after close()."""

    def __init__(self, mesh: Mesh, path, nodal_variables: list[str], title: str = "fec_gb300 results"):
        self.path = str(path)
        self.mesh = mesh
        self.names = list(nodal_variables)
        f = _netcdf()(self.path, "w", version=2)
        self._f = f
        f.api_version = np.float32(8.11)
        f.version = np.float32(8.11)
        f.floating_point_word_size = np.int32(8)
        f.file_size = np.int32(1)
        f.maximum_name_length = np.int32(LEN_STRING - 1)
        f.title = title
        nn, nd = mesh.num_nodes, mesh.num_dimensions
        blocks = mesh.element_block_names
        f.createDimension("time_step", None)  # the record dimension comes first in scipy's writer
        f.createDimension("len_string", LEN_STRING)
        f.createDimension("len_line", 81)
        f.createDimension("four", 4)
        f.createDimension("num_dim", nd)
        f.createDimension("num_nodes", nn)
        f.createDimension("num_elem", mesh.num_elements())
        f.createDimension("num_el_blk", len(blocks))
        t = f.createVariable("time_whole", "d", ("time_step",))
        t.units = "s"
        for d, c in enumerate(("coordx", "coordy", "coordz")[:nd]):
            f.createVariable(c, "d", ("num_nodes",))[:] = mesh.nodal_coords[:, d]
        _put_names(f, "coor_names", "num_dim", ["x", "y", "z"][:nd])
        f.createVariable("eb_status", "i", ("num_el_blk",))[:] = np.ones(len(blocks), dtype=np.int32)
        ids = f.createVariable("eb_prop1", "i", ("num_el_blk",))
        ids[:] = np.arange(1, len(blocks) + 1, dtype=np.int32)
        ids.name = "ID"
        _put_names(f, "eb_names", "num_el_blk", blocks)
        for i, b in enumerate(blocks):
            conn = mesh.element_conns[b]
            f.createDimension(f"num_el_in_blk{i + 1}", conn.shape[0])
            f.createDimension(f"num_nod_per_el{i + 1}", conn.shape[1])
            c = f.createVariable(f"connect{i + 1}", "i", (f"num_el_in_blk{i + 1}", f"num_nod_per_el{i + 1}"))
            c[:] = conn.astype(np.int32)
            c.elem_type = mesh.element_types[b]
        sets = list(mesh.nodeset_nodes)
        if sets:
            f.createDimension("num_node_sets", len(sets))
            f.createVariable("ns_status", "i", ("num_node_sets",))[:] = np.ones(len(sets), dtype=np.int32)
            p = f.createVariable("ns_prop1", "i", ("num_node_sets",))
            p[:] = np.arange(1, len(sets) + 1, dtype=np.int32)
            p.name = "ID"
            _put_names(f, "ns_names", "num_node_sets", sets)
            for i, s in enumerate(sets):
                nodes = mesh.nodeset_nodes[s]
                f.createDimension(f"num_nod_ns{i + 1}", max(1, nodes.size))
                f.createVariable(f"node_ns{i + 1}", "i", (f"num_nod_ns{i + 1}",))[:] = nodes.astype(np.int32)
        if self.names:
            f.createDimension("num_nod_var", len(self.names))
            _put_names(f, "name_nod_var", "num_nod_var", self.names)
            self._vals = [f.createVariable(f"vals_nod_var{k + 1}", "d", ("time_step", "num_nodes"))
                          for k in range(len(self.names))]
        self._time = t

    def write_times(self, time_index: int, time: float) -> None:
        self._time[time_index - 1] = float(time)

    def write_field(self, time_index: int, names, values) -> None:
        """values: (NN,) for one name or (NN, len(names)) (an H1Field's node-major
        layout), host array or device tensor."""
        if hasattr(values, "detach"):
            values = values.detach().cpu().numpy()
        values = np.asarray(values, dtype=np.float64)
        names = [names] if isinstance(names, str) else list(names)
        values = values.reshape(self.mesh.num_nodes, len(names))
        for j, nm in enumerate(names):
            self._vals[self.names.index(nm)][time_index - 1] = values[:, j]

    def close(self) -> None:
        self._f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
