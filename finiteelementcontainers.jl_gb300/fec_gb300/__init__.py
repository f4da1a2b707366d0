"""fec_gb300: the assembly hot path of FiniteElementContainers.jl on GB300.

Host-side mirror of the reference API (meshes, FunctionSpace, DofManager,
DirichletBC, SparseMatrixAssembler, assemble_vector/assemble_stiffness,
residual/stiffness) over the C ABI of libfec_gb300.so, whose sm_103a kernels
do the element quadrature, the gathers and the deterministic scatter."""
from .meshes import StructuredMesh, UnstructuredMesh, Mesh, ArgumentError
from .exodus import ExodusFile, ExodusPostProcessor, read_exodus
from .spaces import FunctionSpace, ScalarFunction, VectorFunction
from . import quadrature
from .quadrature import reference_tables
from .dofs import DofManager, update_dofs
from .bcs import DirichletBC, dirichlet_dofs
from .physics import Poisson, NeoHookean, J2Plasticity, num_fields, num_properties, num_states
from .assemblers import (SparseMatrixAssembler, CSCMatrix, Parameters, create_parameters, update_dofs_bcs,
                         assemble_vector, assemble_stiffness, assemble_matrix, assemble_residual_and_stiffness,
                         residual, stiffness, autotune_report, assemble_matrix_free_action, stiffness_action,
                         hvp, IterativeLinearSolver)
from ._lib import FECError, load as load_library

__all__ = [n for n in dir() if not n.startswith("_")]
