"""The linear solve after assembly (IterativeLinearSolver, src/Solvers.jl:88-152):
conjugate gradients on the GPU-assembled CSC stiffness.  The reference's
poisson.gold (test/poisson/TestPoisson.jl:54-100) through one device solve, a
Neo-Hookean Newton update against a direct solve of the same system, and
bitwise repeatability."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse.linalg as spl

from helpers import rel_err, stretch_field

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("preconditioner", ["none", "jacobi"])
def test_poisson_gold_through_device_solve(fec, preconditioner):
    torch = _torch()
    g = np.load(GOLD / "poisson_quad4.npz")
    mesh = fec.UnstructuredMesh(g["coords"], {"block_1": ("QUAD4", g["conn"])},
                                nodesets={f"nset_{i}": g[f"nset_{i}"] for i in range(1, 5)})
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f"nset_{i}") for i in range(1, 5)]
    asm = fec.SparseMatrixAssembler(fec.ScalarFunction(fec.FunctionSpace(mesh), "u"), device=0)
    p = fec.create_parameters(mesh, asm, fec.Poisson(2 * np.pi ** 2), dirichlet_bcs=bcs)
    solver = fec.IterativeLinearSolver(asm, preconditioner=preconditioner, rtol=1e-13, max_iter=20000)
    Uu = torch.zeros(asm.dof.unknown_dofs.size, dtype=torch.float64, device="cuda")
    solver.solve(Uu, p)
    torch.cuda.synchronize()
    print(preconditioner, "CG iterations", solver.iterations, "relative residual", solver.rel_residual)
    assert solver.rel_residual <= 1e-13
    u = np.zeros(mesh.num_nodes)
    u[asm.dof.unknown_dofs - 1] = Uu.cpu().numpy()
    assert np.abs(u - g["u_gold"]).max() <= 1e-9 * np.abs(g["u_gold"]).max()


def test_poisson_gold_through_exodus_files(fec, tmp_path):
    """The reference's Poisson regression flow end to end through files: the mesh
    written to and read from an Exodus file, the device solve, the solution
    written by the post-processor and read back against poisson.gold
    (test/poisson/TestPoisson.jl:54-100, which compares with exodiff)."""
    torch = _torch()
    g = np.load(GOLD / "poisson_quad4.npz")
    src = fec.UnstructuredMesh(g["coords"], {"block_1": ("QUAD4", g["conn"])},
                               nodesets={f"nset_{i}": g[f"nset_{i}"] for i in range(1, 5)})
    with fec.ExodusPostProcessor(src, tmp_path / "poisson.g", []):
        pass
    mesh = fec.read_exodus(tmp_path / "poisson.g")
    bcs = [fec.DirichletBC("u", lambda X, t: 0.0, nodeset_name=f"nset_{i}") for i in range(1, 5)]
    asm = fec.SparseMatrixAssembler(fec.ScalarFunction(fec.FunctionSpace(mesh), "u"), device=0)
    p = fec.create_parameters(mesh, asm, fec.Poisson(2 * np.pi ** 2), dirichlet_bcs=bcs)
    solver = fec.IterativeLinearSolver(asm, preconditioner="jacobi", rtol=1e-13, max_iter=20000)
    Uu = torch.zeros(asm.dof.unknown_dofs.size, dtype=torch.float64, device="cuda")
    solver.solve(Uu, p)
    torch.cuda.synchronize()
    u = np.zeros(mesh.num_nodes)
    u[asm.dof.unknown_dofs - 1] = Uu.cpu().numpy()
    with fec.ExodusPostProcessor(mesh, tmp_path / "poisson.e", ["u"]) as pp:
        pp.write_times(1, 0.0)
        pp.write_field(1, "u", u)
    with fec.ExodusFile(tmp_path / "poisson.e") as f:
        assert f.nodal_variable_names() == ["u"]
        uo = f.nodal_variable("u", 1)
    assert np.abs(uo - g["u_gold"]).max() <= 1e-9 * np.abs(g["u_gold"]).max()


def test_neohookean_newton_update_matches_direct_solve(fec):
    torch = _torch()
    mesh = fec.StructuredMesh("hex", (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (7, 7, 7))
    asm = fec.SparseMatrixAssembler(fec.VectorFunction(fec.FunctionSpace(mesh), "u"), device=0)
    bcs = [fec.DirichletBC("u_x", lambda X, t: 0.0, nodeset_name="left"),
           fec.DirichletBC("u_y", lambda X, t: 0.0, nodeset_name="bottom"),
           fec.DirichletBC("u_z", lambda X, t: 0.0, nodeset_name="back"),
           fec.DirichletBC("u_x", lambda X, t: 0.02, nodeset_name="right")]
    p = fec.create_parameters(mesh, asm, fec.NeoHookean.from_youngs(1.0, 0.3), dirichlet_bcs=bcs)
    U = stretch_field(mesh.nodal_coords, seed=5, noise=1e-3, diag=(1.01, 0.998, 0.998)).ravel()
    Uu = torch.from_numpy(U[asm.dof.unknown_dofs - 1].copy()).cuda()
    U0 = Uu.clone()
    # the system the solver sees, solved directly
    R, K = fec.assemble_residual_and_stiffness(asm, Uu, p)
    dx = spl.spsolve(K.to_scipy().tocsc(), R.cpu().numpy())
    solver = fec.IterativeLinearSolver(asm, rtol=1e-13)
    solver.solve(Uu, p)
    torch.cuda.synchronize()
    du = (U0 - Uu).cpu().numpy()
    print("CG iterations", solver.iterations, "relative residual", solver.rel_residual, "vs direct", rel_err(du, dx))
    assert max(rel_err(du, dx)[:2]) <= 1e-9   # CG converges normwise
    # repeatable
    Uu2 = U0.clone()
    solver.solve(Uu2, p)
    assert torch.equal(Uu, Uu2)
    # a few Newton iterations reduce the residual
    norms = []
    for _ in range(4):
        R, _ = fec.assemble_residual_and_stiffness(asm, Uu, p)
        norms.append(float(R.norm()))
        solver.solve(Uu, p)
    print("Newton residual norms", norms)
    assert norms[-1] < 1e-6 * norms[0]
