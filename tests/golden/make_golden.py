"""Generates the committed golden fixtures from the reference's own test data.

Run in a checkout that has the reference next to it:
    python tests/golden/make_golden.py /path/to/FiniteElementContainers.jl

Writes
  poisson_quad4.npz   test/poisson/poisson.gold: the 128x128 quad4 mesh
                      (coords, connectivity, the four boundary node sets) and
                      the converged Poisson solution the reference's regression
                      test compares against (test/poisson/TestPoisson.jl:54-100)
  laplace_quad4.npz   test/laplace_with_source/laplace.gold: same mesh, the
                      Laplace-with-source solution (TestLaplace.jl)
  known_answers.json  literal expectations of test/TestMesh.jl (quad4 structured
                      mesh coordinates and connectivity), test/TestFields.jl
                      (multi-block connectivity slices) and
                      test/TestDofManagers.jl (DofManager size on poisson.g)
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np
from scipy.io import netcdf_file

HERE = Path(__file__).resolve().parent


def exodus_quad(path: Path) -> dict:
    g = netcdf_file(str(path), "r", mmap=False)
    v = g.variables
    coords = np.stack([v["coordx"][:], v["coordy"][:]], axis=1).astype(np.float64)
    conn = v["connect1"][:].astype(np.int32)
    nsets = {f"nset_{i}": v[f"node_ns{i}"][:].astype(np.int32) for i in range(1, 5)}
    u = v["vals_nod_var1"][:][-1].astype(np.float64)
    g.close()
    return dict(coords=coords, conn=conn, u_gold=u, **nsets)


def parse_matrix(text: str) -> list[list[float]]:
    rows = [r.strip() for r in text.strip().split(";") if r.strip()]
    return [[float(x) for x in r.split()] for r in rows]


def known_answers(ref: Path) -> dict:
    mesh_src = (ref / "test" / "TestMesh.jl").read_text()
    m = re.search(r'StructuredMesh\("quad", \(0\., 0\.\), \(1\., 1\.\), \(3, 3\)\)\s*coords = mesh\.nodal_coords\s*'
                  r'@test coords ≈ H1Field\(\[(.*?)\]\)\s*@test mesh\.element_conns\["block_1"\] ≈ \[(.*?)\]',
                  mesh_src, re.S)
    quad_coords = parse_matrix(m.group(1))
    quad_conns = parse_matrix(m.group(2))
    fields_src = (ref / "test" / "TestFields.jl").read_text()
    blk = re.search(r"conns_in = \[\s*\[(.*?)\],\s*\[(.*?)\]\s*\]", fields_src, re.S)
    conn1, conn2 = parse_matrix(blk.group(1)), parse_matrix(blk.group(2))
    slices = [(int(b), int(e), int(o), [int(x) for x in vals.split(",")])
              for b, e, o, vals in re.findall(r"@test connectivity\(ref_fe_(\d), conn\.data, (\d+), (\d+)\) == \[([\d, ]+)\]",
                                              fields_src)]
    dof_src = (ref / "test" / "TestDofManagers.jl").read_text()
    size = re.search(r"@test size\(dof1\) == \((\d+), (\d+)\)", dof_src)
    return dict(
        structured_quad4_3x3=dict(coords=quad_coords, conns=quad_conns),
        connectivity=dict(block_1=conn1, block_2=conn2, slices=slices),
        dofmanager_vector_poisson_g=[int(size.group(1)), int(size.group(2))],
    )


def main(ref: Path) -> None:
    p = exodus_quad(ref / "test" / "poisson" / "poisson.gold")
    np.savez_compressed(HERE / "poisson_quad4.npz", **p)
    lap = exodus_quad(ref / "test" / "laplace_with_source" / "laplace.gold")
    np.savez_compressed(HERE / "laplace_quad4.npz", u_gold=lap["u_gold"])
    (HERE / "known_answers.json").write_text(json.dumps(known_answers(ref), indent=1))
    print("wrote", sorted(x.name for x in HERE.iterdir() if x.suffix in (".npz", ".json")))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/FiniteElementContainers.jl")
    main(Path(sys.argv[1]))
