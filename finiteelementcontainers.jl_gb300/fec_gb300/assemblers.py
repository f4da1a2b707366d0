"""SparseMatrixAssembler and the assembly entry points, over libfec_gb300.so.

Mirrors src/assemblers/SparseMatrixAssembler.jl, Vector.jl, Matrix.jl and the
residual/stiffness accessors of Assemblers.jl for the default configuration
(CSC, non-condensed, return-value physics methods).  Julia's in-place `!`
names lose the bang: assemble_vector!(asm, residual, Uu, p) becomes
assemble_vector(asm, residual, Uu, p).

Device memory, streams and the host<->device copies use torch; every
assembly FLOP runs in the library's sm_103a kernels.  There is no CPU
fallback: without the library (or without a GPU) these calls raise."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .bcs import dirichlet_dofs
from .dofs import DofManager, update_dofs
from .meshes import ELEMENT_IDS
from .physics import AbstractPhysics
from .spaces import FunctionSpace

PRECISIONS = {"fp64": _lib.FEC_FP64, "fp32_element": _lib.FEC_FP32_ELEMENT}


def _torch():
    import torch
    return torch


class CSCMatrix:
    """Sparse CSC matrix over unknowns: 1-based int64 colptr/rowval on the host
    (SparseMatrixCSC layout) and the values on the device (CuSparseMatrixCSC's nzval)."""

    def __init__(self, n: int, colptr: np.ndarray, rowval: np.ndarray, nzval):
        self.shape = (n, n)
        self.colptr = colptr
        self.rowval = rowval
        self.nzval = nzval

    @property
    def nnz(self) -> int:
        return int(self.rowval.size)

    def to_scipy(self):
        import scipy.sparse as sp
        vals = self.nzval.detach().cpu().numpy() if hasattr(self.nzval, "detach") else np.asarray(self.nzval)
        return sp.csc_matrix((vals, self.rowval - 1, self.colptr - 1), shape=self.shape)


class SparseMatrixAssembler:
    """SparseMatrixAssembler(var; sparse_matrix_type=:csc, use_condensed=false)
    (src/assemblers/SparseMatrixAssembler.jl:64-133).

    device: CUDA device index, or -1 for a host-only assembler that can build
    the pattern (colptr/rowval) but not assemble values.
    symbolic: "host" builds the pattern and its maps on the host threads
    (fec_pattern_build), "device" with kernels (fec_pattern_build_device); both
    give the same pattern and maps."""

    def __init__(self, var_or_dof, *, sparse_matrix_type: str = "csc", use_condensed: bool = False,
                 use_inplace_methods: bool = False, device: int = 0, precision: str = "fp64",
                 symbolic: str = "host"):
        if sparse_matrix_type != "csc":
            raise NotImplementedError(f"sparse_matrix_type={sparse_matrix_type!r}: the accelerated path builds CSC")
        if use_condensed:
            raise NotImplementedError("use_condensed=true is not on the accelerated path")
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        if symbolic not in ("host", "device"):
            raise ValueError("symbolic must be 'host' or 'device'")
        if symbolic == "device" and device < 0:
            raise ValueError("symbolic='device' needs a CUDA device")
        self.symbolic = symbolic
        self.dof = var_or_dof if isinstance(var_or_dof, DofManager) else DofManager(var_or_dof)
        self.fspace: FunctionSpace = self.dof.var.fspace
        self.use_inplace_methods = use_inplace_methods
        self.precision = precision
        self.device = device
        self._lib = _lib.load()
        h = C.c_void_p()
        st = self._lib.fec_ctx_create(device, C.byref(h))
        if st != _lib.FEC_OK:
            raise _lib.FECError(st, _lib.last_error(self._lib, None))
        self._ctx = h
        fs = self.fspace
        coords = np.ascontiguousarray(fs.coords, dtype=np.float64)
        types = fs.element_type_ids()
        self._call("fec_mesh_set", fs.num_dimensions, fs.num_nodes, _lib.ptr(coords), len(types), _lib.ptr(types),
                   _lib.ptr(fs.block_num_elems), _lib.ptr(fs.conn_data))
        self.set_reference_tables()
        self._physics_key = None
        self._push_dofs()

    # -- plumbing ---------------------------------------------------------------
    def _call(self, name, *args):
        _lib.check(self._lib, self._ctx, getattr(self._lib, name)(self._ctx, *args))

    def __del__(self):
        ctx = getattr(self, "_ctx", None)
        if ctx is not None and ctx.value:
            self._lib.fec_ctx_destroy(ctx)
            self._ctx = None

    def _push_dofs(self):
        dtu = np.ascontiguousarray(self.dof.dof_to_unknown, dtype=np.int64)
        self._call("fec_dofs_set", self.dof.nf, _lib.ptr(dtu), int(self.dof.unknown_dofs.size))
        self._pattern_dirty = True
        self._csc_host = None
        self.residual_unknowns = None
        self.stiffness_nzval = None

    def _ensure_pattern(self):
        if self._pattern_dirty:
            nnz = C.c_int64()
            if self.symbolic == "device":
                torch = _torch()
                with torch.cuda.device(self.device):
                    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
                self._call("fec_pattern_build_device", C.byref(nnz), s)
            else:
                self._call("fec_pattern_build", C.byref(nnz))
            self.nnz = int(nnz.value)
            self._pattern_dirty = False
        return self.nnz

    def _torch_device(self):
        return f"cuda:{self.device}"

    # -- reference API -------------------------------------------------------------
    def pattern(self) -> tuple[np.ndarray, np.ndarray]:
        """1-based (colptr, rowval) of the CSC stiffness over unknowns."""
        self._ensure_pattern()
        if self._csc_host is None:
            n = int(self.dof.unknown_dofs.size)
            colptr = np.empty(n + 1, dtype=np.int64)
            rowval = np.empty(self.nnz, dtype=np.int64)
            self._call("fec_pattern_get", _lib.ptr(colptr), _lib.ptr(rowval))
            self._csc_host = (colptr, rowval)
        return self._csc_host

    def set_reference_tables(self, tables=None) -> None:
        """Hands each block's quadrature rule and shape-function tables to the
        library (fec_block_reference_set): the function space's ReferenceFEs, or
        `tables`, a list of (N, dN, w) per block."""
        tables = self.fspace.ref_fes if tables is None else tables
        for b, (N, dN, w) in enumerate(tables, start=1):
            N = np.ascontiguousarray(N, dtype=np.float64)
            dN = np.ascontiguousarray(dN, dtype=np.float64)
            w = np.ascontiguousarray(w, dtype=np.float64)
            self._call("fec_block_reference_set", b, int(w.size), _lib.ptr(N), _lib.ptr(dN), _lib.ptr(w))

    def reference_tables(self, block: int):
        """(N, dN, w) block `block` (1-based) is assembled with (fec_block_reference_get)."""
        fs = self.fspace
        nq = C.c_int()
        self._call("fec_block_reference_get", block, C.byref(nq), None, None, None)
        nnpe, dim = int(fs.nepes[block - 1]), fs.num_dimensions
        N = np.empty((nq.value, nnpe)); dN = np.empty((nq.value, nnpe, dim)); w = np.empty(nq.value)
        self._call("fec_block_reference_get", block, C.byref(nq), _lib.ptr(N), _lib.ptr(dN), _lib.ptr(w))
        return N, dN, w

    def set_single_launch(self, on: bool = True) -> None:
        """Run every element block of an FP64 Neo-Hookean/J2 system (hex8, tet4,
        tet10, hex27 blocks) in one persistent launch (fec_set_single_launch)."""
        self._call("fec_set_single_launch", 1 if on else 0)

    def pattern_device(self):
        """1-based (colptr, rowval) of the CSC stiffness as int64 device tensors,
        filled by a kernel (for a CuSparse-style matrix on the device)."""
        torch = _torch()
        self._ensure_pattern()
        n = int(self.dof.unknown_dofs.size)
        dev = self._torch_device()
        colptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
        rowval = torch.empty(self.nnz, dtype=torch.int64, device=dev)
        with torch.cuda.device(self.device):
            s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._call("fec_pattern_get_device", _lib.ptr(colptr), _lib.ptr(rowval), s)
        return colptr, rowval

    def create_field(self):
        return _torch().zeros(len(self.dof), dtype=_torch().float64, device=self._torch_device())

    def create_unknowns(self):
        return _torch().zeros(self.dof.unknown_dofs.size, dtype=_torch().float64, device=self._torch_device())

    def last_launch_count(self) -> int:
        return int(self._lib.fec_last_launch_count(self._ctx))

    def set_profiling(self, on: bool) -> None:
        self._call("fec_set_profiling", int(bool(on)))

    def kernel_times(self) -> list[tuple[str, float]]:
        """(name, ms) of each launch of the last update+assemble pair (profiling on)."""
        ms = (C.c_float * 64)()
        names = C.create_string_buffer(1024)
        n = self._lib.fec_kernel_times(self._ctx, ms, 64, names, 1024)
        if n < 0:
            _lib.check(self._lib, self._ctx, n)
        labels = names.value.decode().split(",") if n else []
        return [(labels[i], float(ms[i])) for i in range(n)]


def update_dofs_bcs(asm: SparseMatrixAssembler, dirichlet_bcs) -> None:
    """update_dofs!(asm, dirichlet_bcs, periodic_bcs) (SparseMatrixAssembler.jl:228-274)."""
    ddofs = dirichlet_dofs(dirichlet_bcs, asm.fspace.mesh, asm.dof)
    update_dofs(asm.dof, ddofs)
    asm._push_dofs()


class Parameters:
    """The parts of Parameters (src/Parameters.jl) the assembly reads: time,
    nodal field U (device), per-block physics/properties, state old/new
    ((NS, NQ, NE) per block, concatenated) and Dirichlet values."""

    def __init__(self, mesh, asm: SparseMatrixAssembler, physics, props=None, *, dirichlet_bcs=(), t: float = 0.0,
                 dt: float = 0.0):
        torch = _torch()
        nb = asm.fspace.num_blocks()
        if isinstance(physics, AbstractPhysics):
            physics = {name: physics for name in asm.fspace.block_names}
        self.physics = [physics[name] for name in asm.fspace.block_names]
        if props is None:
            props = {name: ph.create_properties() for name, ph in zip(asm.fspace.block_names, self.physics)}
        elif not isinstance(props, dict):
            props = {name: props for name in asm.fspace.block_names}
        self.props = [np.ascontiguousarray(props[name], dtype=np.float64) for name in asm.fspace.block_names]
        for ph in self.physics:
            if ph.NF != asm.dof.nf:
                raise ValueError(f"physics {type(ph).__name__} has {ph.NF} fields but the function has {asm.dof.nf}")
        dev = asm._torch_device()
        self.t, self.dt = float(t), float(dt)
        self.dirichlet_bcs = list(dirichlet_bcs)
        update_dofs_bcs(asm, self.dirichlet_bcs)
        self.field = torch.zeros(len(asm.dof), dtype=torch.float64, device=dev)
        self.field_old = torch.zeros_like(self.field)
        sizes = []
        for b, (ph, (nq, ne)) in enumerate(zip(self.physics, asm.fspace.block_quadrature_sizes())):
            s0 = ph.create_initial_state()
            sizes.append(np.tile(s0, nq * ne))
        init = np.concatenate(sizes) if sizes else np.zeros(0)
        self.state_old = torch.as_tensor(init, dtype=torch.float64).to(dev)
        self.state_new = self.state_old.clone()
        self._mesh = mesh
        self._asm = asm
        self.update_bc_values()
        assert nb == len(self.physics)

    def update_bc_values(self):
        """update_bc_values!(dirichlet_bcs, X, t): evaluate each BC at its nodes."""
        torch = _torch()
        dofs, vals = [], []
        X = self._asm.fspace.coords
        for bc in self.dirichlet_bcs:
            d, nodes = bc.dofs_and_nodes(self._mesh, self._asm.dof)
            dofs.append(d)
            vals.append(np.array([bc.func(X[n - 1], self.t) for n in nodes], dtype=np.float64))
        dev = self._asm._torch_device()
        if dofs:
            d = np.concatenate(dofs)
            v = np.concatenate(vals)
            self.bc_dofs = torch.as_tensor(d, dtype=torch.int64).to(dev)
            self.bc_vals = torch.as_tensor(v, dtype=torch.float64).to(dev)
        else:
            self.bc_dofs = torch.zeros(0, dtype=torch.int64, device=dev)
            self.bc_vals = torch.zeros(0, dtype=torch.float64, device=dev)

    def swap_states(self):
        """state_old <- state_new after a converged step (the reference leaves
        this to downstream applications)."""
        self.state_old, self.state_new = self.state_new, self.state_old


def create_parameters(mesh, asm, physics, props=None, *, dirichlet_bcs=(), t: float = 0.0, dt: float = 0.0):
    """create_parameters(mesh, asm, physics, props; dirichlet_bcs) (src/Parameters.jl:288-302)."""
    return Parameters(mesh, asm, physics, props, dirichlet_bcs=dirichlet_bcs, t=t, dt=dt)


# -- physics-method markers (the Julia generic functions residual/stiffness) ---------------------

def residual(obj, *args):
    """residual(asm): the assembled residual over unknowns (Assemblers.jl:347-371).
    Passed as the function argument of assemble_vector it selects the physics'
    residual, which runs on the device."""
    if isinstance(obj, SparseMatrixAssembler):
        if obj.residual_unknowns is None:
            obj.residual_unknowns = obj.create_unknowns()
        return obj.residual_unknowns
    raise TypeError("physics residuals run inside the device kernels; pass `residual` to assemble_vector")


def stiffness(obj, *args):
    """stiffness(asm): the assembled CSC tangent over unknowns (Assemblers.jl:376-388)."""
    if isinstance(obj, SparseMatrixAssembler):
        colptr, rowval = obj.pattern()
        if obj.stiffness_nzval is None:
            obj.stiffness_nzval = _torch().zeros(obj.nnz, dtype=_torch().float64, device=obj._torch_device())
        return CSCMatrix(int(obj.dof.unknown_dofs.size), colptr, rowval, obj.stiffness_nzval)
    raise TypeError("physics tangents run inside the device kernels; pass `stiffness` to assemble_stiffness")


def _as_device_unknowns(asm, Uu):
    torch = _torch()
    dev = asm._torch_device()
    if isinstance(Uu, np.ndarray):
        return torch.from_numpy(np.ascontiguousarray(Uu, dtype=np.float64)).to(dev, non_blocking=True)
    if Uu.device.type != "cuda":
        return Uu.to(dev, dtype=torch.float64, non_blocking=True)
    if Uu.dtype != torch.float64 or not Uu.is_contiguous():
        raise TypeError("Uu must be a contiguous float64 tensor")
    return Uu


def _prepare(asm: SparseMatrixAssembler, Uu, p: Parameters):
    """Physics set-up (once per change) and _update_for_assembly! (src/Parameters.jl:404-413)."""
    torch = _torch()
    asm._ensure_pattern()
    key = tuple((ph.ID, pr.tobytes(), id(getattr(ph, "closure", None))) for ph, pr in zip(p.physics, p.props))
    if key != asm._physics_key:
        for b, (ph, pr) in enumerate(zip(p.physics, p.props), start=1):
            asm._call("fec_physics_set", b, ph.ID, _lib.ptr(pr), int(pr.size))
            if hasattr(ph, "install"):   # physics that carry device data (the learned closure)
                ph.install(asm)
        asm._physics_key = key
    n_u = int(asm.dof.unknown_dofs.size)
    Uu_d = _as_device_unknowns(asm, Uu)
    if Uu_d.numel() != n_u:
        raise ValueError(f"Uu has {Uu_d.numel()} entries, expected {n_u}")
    stream = C.c_void_p(torch.cuda.current_stream(asm.device).cuda_stream)
    asm._call("fec_update_field", _lib.ptr(p.field), _lib.ptr(Uu_d), int(p.bc_dofs.numel()),
              _lib.ptr(p.bc_dofs) if p.bc_dofs.numel() else None,
              _lib.ptr(p.bc_vals) if p.bc_vals.numel() else None, stream)
    return stream


def _check_out(asm: SparseMatrixAssembler, t, n: int, name: str):
    torch = _torch()
    if not (isinstance(t, torch.Tensor) and t.dtype == torch.float64 and t.is_contiguous() and t.numel() == n
            and t.device == torch.device(asm._torch_device())):
        raise ValueError(f"out {name} must be a contiguous float64 tensor of {n} entries on {asm._torch_device()}")
    return t


def _assemble(asm: SparseMatrixAssembler, want: int, Uu, p: Parameters, precision: str | None, out=None):
    stream = _prepare(asm, Uu, p)
    if out is None:
        R = residual(asm) if want & _lib.FEC_WANT_RESIDUAL else None
        K = stiffness(asm) if want & _lib.FEC_WANT_STIFFNESS else None
    else:
        colptr, rowval = asm.pattern()
        R = _check_out(asm, out[0], int(asm.dof.unknown_dofs.size), "residual")
        K = CSCMatrix(int(asm.dof.unknown_dofs.size), colptr, rowval, _check_out(asm, out[1], asm.nnz, "nzval"))
    has_state = any(ph.NS for ph in p.physics)
    asm._call("fec_assemble", want, PRECISIONS[precision or asm.precision], p.t, p.dt, _lib.ptr(p.field),
              _lib.ptr(p.field_old), _lib.ptr(p.state_old) if has_state else None,
              _lib.ptr(p.state_new) if has_state else None, _lib.ptr(R), _lib.ptr(K.nzval) if K else None, stream)
    return R, K


def assemble_vector(asm: SparseMatrixAssembler, func, Uu, p: Parameters, *, precision: str | None = None):
    """assemble_vector!(asm, residual, Uu, p) (src/assemblers/Vector.jl:4-20)."""
    if func is not residual:
        raise NotImplementedError("assemble_vector supports the physics `residual` method")
    _assemble(asm, _lib.FEC_WANT_RESIDUAL, Uu, p, precision)


def assemble_stiffness(asm: SparseMatrixAssembler, func, Uu, p: Parameters, *, precision: str | None = None):
    """assemble_stiffness!(asm, stiffness, Uu, p) (src/assemblers/Matrix.jl:12-21)."""
    if func is not stiffness:
        raise NotImplementedError("assemble_stiffness supports the physics `stiffness` method")
    _assemble(asm, _lib.FEC_WANT_STIFFNESS, Uu, p, precision)


assemble_matrix = assemble_stiffness


def assemble_residual_and_stiffness(asm: SparseMatrixAssembler, Uu, p: Parameters, *, precision: str | None = None,
                                    check_finite: bool = False, out=None):
    """One fused pass producing both residual(asm) and stiffness(asm), the pair a
    Newton iteration assembles (src/Solvers.jl:128-153).  check_finite raises
    FECError (FEC_ERR_NONFINITE) when an output holds NaN/Inf (synchronises).
    out = (R, nzval): device float64 tensors (unknowns, nnz) the pass writes
    instead of the assembler's own arrays -- a caller that reads one pair back
    while the next pass writes the other alternates two."""
    R, K = _assemble(asm, _lib.FEC_WANT_RESIDUAL | _lib.FEC_WANT_STIFFNESS, Uu, p, precision, out)
    if check_finite:
        check_finite_outputs(asm, R, K)
    return R, K


def check_finite_outputs(asm: SparseMatrixAssembler, R=None, K=None) -> None:
    """Raise FECError (FEC_ERR_NONFINITE) if the residual or the stiffness values hold NaN/Inf."""
    torch = _torch()
    bad = C.c_int64(-1)
    stream = C.c_void_p(torch.cuda.current_stream(asm.device).cuda_stream)
    asm._call("fec_check_finite", _lib.ptr(R), _lib.ptr(K.nzval) if K is not None else None, C.byref(bad), stream)


def stiffness_action(*_):
    """Marker of the physics' tangent action (stiffness_action in the reference)."""
    raise TypeError("stiffness_action is a marker for assemble_matrix_free_action")


def assemble_matrix_free_action(asm: SparseMatrixAssembler, func, Uu, Vu, p: Parameters, *,
                                precision: str | None = None):
    """assemble_matrix_free_action!(asm, stiffness_action, Uu, Vu, p)
    (src/assemblers/MatrixAction.jl:9-77): K v over the unknowns without forming
    K; read it with hvp(asm).  Dirichlet components of the direction are zero."""
    torch = _torch()
    if func is not stiffness_action:
        raise NotImplementedError("assemble_matrix_free_action supports the physics `stiffness_action` method")
    stream = _prepare(asm, Uu, p)
    n_u = int(asm.dof.unknown_dofs.size)
    Vu_d = _as_device_unknowns(asm, Vu)
    if Vu_d.numel() != n_u:
        raise ValueError(f"Vu has {Vu_d.numel()} entries, expected {n_u}")
    if getattr(asm, "_hvp", None) is None or asm._hvp.numel() != n_u:
        asm._hvp = torch.empty(n_u, dtype=torch.float64, device=asm._torch_device())
    has_state = any(ph.NS for ph in p.physics)
    asm._call("fec_assemble_action", PRECISIONS[precision or asm.precision], p.t, p.dt, _lib.ptr(p.field),
              _lib.ptr(p.state_old) if has_state else None, _lib.ptr(Vu_d), _lib.ptr(asm._hvp), stream)
    return asm._hvp


def hvp(asm: SparseMatrixAssembler, Vu=None):
    """hvp(asm, v) (src/assemblers/Assemblers.jl:310-324): the last matrix-free action
    over the unknowns (a device view)."""
    if getattr(asm, "_hvp", None) is None:
        raise RuntimeError("hvp before assemble_matrix_free_action")
    return asm._hvp


class IterativeLinearSolver:
    """IterativeLinearSolver (src/Solvers.jl:88-152) on the device: solve! assembles
    the residual and the stiffness (one fused pass), solves K x = R by conjugate
    gradients on the assembled CSC (fec_cg_solve), and updates Uu -= x.
    preconditioner "none" is the reference's Krylov CG; "jacobi" scales by the
    diagonal."""

    def __init__(self, assembler: SparseMatrixAssembler, *, preconditioner: str = "jacobi", rtol: float = 1e-10,
                 max_iter: int = 10000):
        if preconditioner not in ("none", "jacobi"):
            raise ValueError("preconditioner is 'none' or 'jacobi'")
        self.assembler = assembler
        self.preconditioner = preconditioner
        self.rtol, self.max_iter = float(rtol), int(max_iter)
        self.iterations, self.rel_residual = 0, float("nan")
        self.dUu = None

    def solve(self, Uu, p: Parameters):
        """solve!(solver, Uu, p): one Newton update of the device unknowns Uu in place."""
        torch = _torch()
        asm = self.assembler
        R, K = assemble_residual_and_stiffness(asm, Uu, p)
        if self.dUu is None or self.dUu.numel() != R.numel():
            self.dUu = torch.zeros_like(R)
        else:
            self.dUu.zero_()
        it, rr = C.c_int(0), C.c_double(0.0)
        stream = C.c_void_p(torch.cuda.current_stream(asm.device).cuda_stream)
        asm._call("fec_cg_solve", _lib.ptr(K.nzval), _lib.ptr(R), _lib.ptr(self.dUu), self.max_iter, self.rtol,
                  1 if self.preconditioner == "jacobi" else 0, C.byref(it), C.byref(rr), stream)
        self.iterations, self.rel_residual = it.value, rr.value
        Uu.sub_(self.dUu)
        return Uu


__all__ = ["SparseMatrixAssembler", "CSCMatrix", "Parameters", "create_parameters", "update_dofs_bcs",
           "assemble_vector", "assemble_stiffness", "assemble_matrix", "assemble_residual_and_stiffness",
           "assemble_matrix_free_action", "stiffness_action", "hvp", "residual", "stiffness", "ELEMENT_IDS",
           "IterativeLinearSolver", "check_finite_outputs"]


def autotune_report() -> list[str]:
    """Launch configurations chosen by the library's autotuner (one line per
    kernel family and problem-size bucket, with every candidate's time)."""
    lib = _lib.load()
    buf = C.create_string_buffer(1 << 16)
    lib.fec_autotune_report(buf, len(buf))
    return [ln for ln in buf.value.decode().splitlines() if ln]
