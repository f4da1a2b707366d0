/*
 * fec_gb300.h -- C ABI of the GB300 (sm_103a) assembly library libfec_gb300.so.
 *
 * The library replaces the KernelAbstractions/Atomix device path of
 * FiniteElementContainers.jl's SparseMatrixAssembler: per-element quadrature of
 * the physics residual and tangent, the DOF/coordinate gather through the
 * DofManager and FunctionSpace connectivity, and the deterministic scatter into
 * the global residual over unknowns and the CSC nzval.
 *
 * Conventions (all follow the reference so that its arrays pass unchanged):
 *   - integer inputs are 1-based int64 (Julia Int), as the reference stores them;
 *   - coordinates and nodal fields are interleaved, field[(node-1)*NF + d]
 *     (H1Field, src/Fields.jl:36-40, 237-254);
 *   - connectivity is the flat concatenation of per-block NNPE x NE
 *     column-major matrices (Connectivity, src/Fields.jl:129-160);
 *   - colptr/rowval come back 1-based int64, ready for SparseMatrixCSC;
 *   - pointers named *_dev are device pointers owned by the caller (a CuArray's
 *     pointer(x) in Julia, a torch tensor's data_ptr() in Python); everything
 *     else is host memory.  The library owns connectivity, maps and workspaces
 *     inside the context and frees them in fec_ctx_destroy.
 *   - every call returns FEC_OK (0) or a negative fec_status; fec_last_error
 *     gives the message.  Nothing aborts or traps.
 *   - device work is ordered on the caller's stream (cudaStream_t passed as
 *     void*; NULL = legacy default stream).  One context per host thread.
 */
#ifndef FEC_GB300_H
#define FEC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fec_ctx fec_ctx;

/* status codes */
enum {
  FEC_OK = 0,
  FEC_ERR_ARG = -1,       /* bad argument (null, size, range) */
  FEC_ERR_STATE = -2,     /* call out of order (e.g. assemble before pattern) */
  FEC_ERR_CUDA = -3,      /* a CUDA runtime call failed */
  FEC_ERR_UNSUPPORTED = -4,/* element/physics combination not built */
  FEC_ERR_NONFINITE = -5, /* NaN/Inf found in an assembled output */
  FEC_ERR_DEVICE = -6     /* a kernel reported an error status */
};

/* element types: the reference's juliac-safe ids where it has one
 * (src/FunctionSpaces.jl:48-62); HEX27 is this library's own */
enum { FEC_HEX8 = 1, FEC_QUAD4 = 2, FEC_TET4 = 6, FEC_TET10 = 7, FEC_HEX27 = 8 };

/* physics plugins; the reference selects them by Julia dispatch on
 * AbstractPhysics{NF,NP,NS} (src/Physics.jl:1-57), which cannot cross a C ABI,
 * so here they are an enum plus a property block */
enum {
  FEC_PHYS_POISSON = 1,    /* NF=1; props[0] = source amplitude a, f(X) = a prod_d sin(pi X_d) */
  FEC_PHYS_NEOHOOKEAN = 2, /* NF=3; props = {bulk K, shear G} */
  FEC_PHYS_J2 = 3,         /* NF=3, NS=7; props = {E, nu, sigma_y, H} */
  FEC_PHYS_J2_MLP = 4      /* J2 with the learned closure at plastic points (hex8, FEC_FP32_ELEMENT);
                              props as FEC_PHYS_J2; needs fec_closure_set */
};

/* arithmetic of the element kernels */
enum {
  FEC_FP64 = 0,         /* FP64 throughout */
  FEC_FP32_ELEMENT = 1  /* per-element kinematics/stress/tangent in FP32, Jacobian
                           det/inverse and the global accumulation in FP64 */
};

/* what fec_assemble writes */
enum { FEC_WANT_RESIDUAL = 1, FEC_WANT_STIFFNESS = 2 };

/* Context ------------------------------------------------------------------ */

/* Replaces: the device move of an assembler, asm |> cuda
 * (ext/CUDAExt.jl:8-10, src/Utils.jl:286-291).  device = -1 makes a host-only
 * context: mesh, DOF and pattern calls work, kernel calls return FEC_ERR_STATE. */
int fec_ctx_create(int device, fec_ctx** out);
int fec_ctx_destroy(fec_ctx* ctx);
/* Copies the last error message of ctx (or of the last failed create when
 * ctx is NULL) into buf; returns the last status. */
int fec_last_error(const fec_ctx* ctx, char* buf, size_t len);

/* Mesh / FunctionSpace ------------------------------------------------------ */

/* Replaces: FunctionSpace(mesh, H1Field, Lagrange) connectivity + coordinates
 * (src/FunctionSpaces.jl:104-126, src/Fields.jl:129-188).
 * coords: dim x num_nodes interleaved; conn: flat 1-based, block b holding
 * nnpe(elem_types[b]) * block_num_elems[b] entries. */
int fec_mesh_set(fec_ctx* ctx, int dim, int64_t num_nodes, const double* coords, int num_blocks,
                 const int32_t* elem_types, const int64_t* block_num_elems, const int64_t* conn);

/* Replaces: the block's ReferenceFE (src/FunctionSpaces.jl:104-126) -- its
 * quadrature rule and the shape-function values and reference-coordinate
 * gradients at the points, the interpolants _cell_interpolants hands to the
 * physics (src/assemblers/Assemblers.jl:129-131).  The caller passes the tables
 * its own ReferenceFE holds, so the assembled values follow the caller's rule
 * (GaussLobattoLegendre, the reference's default q_type at
 * src/FunctionSpaces.jl:187, or any other).  Host arrays, row-major:
 *   N  [num_q][nnpe]       shape-function values at the points
 *   dN [num_q][nnpe][dim]  their gradients in reference coordinates
 *   w  [num_q]             quadrature weights
 * num_q must be the point count the block's kernels are built for (HEX8 8,
 * QUAD4 4, TET4 1, TET10 4, HEX27 27; FEC_ERR_UNSUPPORTED otherwise).  A block
 * whose tables are never set uses the library's own: the Gauss-Legendre tensor
 * rule with 2 points per direction (HEX8, QUAD4) or 3 (HEX27), and the 1- and
 * 4-point rules of TET4 and TET10.  fec_mesh_set resets every block to those.
 * Synchronous; do not call it while an assembly of this context is in flight. */
int fec_block_reference_set(fec_ctx* ctx, int block, int num_q, const double* N, const double* dN,
                            const double* w);
/* The tables block `block` currently uses (any output may be NULL; num_q gets
 * the point count, N/dN/w need room for the sizes above). */
int fec_block_reference_get(const fec_ctx* ctx, int block, int* num_q, double* N, double* dN, double* w);

/* Per-block physics and properties (the (physics, props) pair that
 * foreach_block hands to _assemble_block!, src/Utils.jl:171-189).  Poisson: the
 * source amplitude; Neo-Hookean: bulk and shear modulus; J2 and J2-MLP: E, nu,
 * sigma_y, H -- the library keeps constants derived from these in property
 * slots 4-7 (values passed there are replaced). */
int fec_physics_set(fec_ctx* ctx, int block, int physics, const double* props, int num_props);

/* DofManager ---------------------------------------------------------------- */

/* Replaces: update_dofs!(dof, dirichlet_dofs, ...) (src/DofManagers.jl:227-298)
 * as consumed by the assembler.  dof_to_unknown has num_fields * num_nodes
 * entries: the 1-based unknown index of each dof, or -1 for a Dirichlet dof;
 * unknowns must be numbered in increasing dof order, as the reference does. */
int fec_dofs_set(fec_ctx* ctx, int num_fields, const int64_t* dof_to_unknown, int64_t num_unknowns);

/* Sparsity pattern ---------------------------------------------------------- */

/* Replaces: SparseMatrixPattern + _update_dofs! (src/assemblers/SparsityPatterns.jl:53-117,
 * 160-231) together with the colptr/rowval half of SparseArrays.sparse!
 * (:301-308).  Builds the CSC pattern over unknowns and the element -> nzval
 * maps; returns the number of stored entries. */
int fec_pattern_build(fec_ctx* ctx, int64_t* nnz_out);
/* Copies the 1-based colptr (num_unknowns + 1) and rowval (nnz) to host. */
int fec_pattern_get(const fec_ctx* ctx, int64_t* colptr, int64_t* rowval);
/* The symbolic phase on the device (SparseMatrixPattern + _update_dofs!,
 * src/assemblers/SparsityPatterns.jl:53-231): the same pattern, maps and nnz as
 * fec_pattern_build, formed by kernels on `stream` (the call waits for them).
 * FEC_ERR_UNSUPPORTED for more than 16 element blocks or a node whose adjacent
 * elements hold more than 2048 nodes. */
int fec_pattern_build_device(fec_ctx* ctx, int64_t* nnz_out, void* stream);
/* FP64 Neo-Hookean / J2 systems of two to four blocks of hex8, tet4, tet10 or
 * hex27 elements (one physics): on != 0 runs every element block in ONE
 * persistent launch (a work list of per-type tiles) instead of one launch per
 * block; the assembled values are bitwise the same.  Other systems keep one
 * launch per block.  No counterpart in the reference, which launches one
 * kernel per block from foreach_block (src/Utils.jl:171-189). */
int fec_set_single_launch(fec_ctx* ctx, int on);
/* 1-based colptr (n_unknowns + 1) and rowval (nnz) written into DEVICE buffers
 * on `stream` (the colptr/rowval of sparse!, SparsityPatterns.jl:301-308). */
int fec_pattern_get_device(const fec_ctx* ctx, int64_t* colptr_dev, int64_t* rowval_dev, void* stream);

/* Field update -------------------------------------------------------------- */

/* Replaces: update_field_dirichlet_bcs! + update_field_unknowns!
 * (src/bcs/DirichletBCs.jl:411-418, src/DofManagers.jl:349-411).
 * U_dev[bc_dofs[i]-1] = bc_vals[i];  U_dev[unknown_dofs[k]-1] = Uu_dev[k].
 * bc_dofs_dev/bc_vals_dev may be NULL when num_bc == 0. */
int fec_update_field(fec_ctx* ctx, double* U_dev, const double* Uu_dev, int64_t num_bc, const int64_t* bc_dofs_dev,
                     const double* bc_vals_dev, void* stream);

/* Assembly ------------------------------------------------------------------ */

/* Replaces: assemble_vector! + residual(asm) and assemble_stiffness!/
 * assemble_matrix! + stiffness(asm) (src/assemblers/Vector.jl:4-74,
 * src/assemblers/Matrix.jl:12-75, src/assemblers/Assemblers.jl:347-388, 402-432),
 * non-condensed, CSC.
 *   U_dev        full nodal field (NF * num_nodes), already updated
 *   U_old_dev    previous field (may be NULL; no physics here reads it)
 *   state_*_dev  per block (NS, NQ, NE) column-major, blocks concatenated; NULL when NS = 0
 *   R_u_dev      residual over unknowns (num_unknowns), written when want & FEC_WANT_RESIDUAL
 *   nzval_dev    CSC values (nnz), written when want & FEC_WANT_STIFFNESS
 * Contributions to one output entry are summed in increasing element order,
 * the order SparseArrays.sparse! combines the reference's element-ordered COO
 * entries, so repeated calls give bitwise-identical results. */
int fec_assemble(fec_ctx* ctx, int want, int precision, double t, double dt, const double* U_dev,
                 const double* U_old_dev, const double* state_old_dev, double* state_new_dev, double* R_u_dev,
                 double* nzval_dev, void* stream);

/* Matrix-free tangent action: Kv_u = K_uu Vu without forming K.  U is the full
 * field (after fec_update_field), Vu the direction over the unknowns (its
 * Dirichlet components are zero), Kv_u the product over the unknowns (device,
 * caller-owned).  Element contributions are summed over quadrature points in
 * point order and over elements in element order (deterministic).  The state is
 * read, never written.  Replaces assemble_matrix_free_action!(asm,
 * stiffness_action, Uu, Vu, p) followed by hvp(asm, Vu)
 * (src/assemblers/MatrixAction.jl:9-77, src/assemblers/Assemblers.jl:310-324).
 * Poisson, Neo-Hookean and J2 on hex8/tet4/tet10/hex27 (quad4 for Poisson). */
int fec_assemble_action(fec_ctx* ctx, int precision, double t, double dt, const double* U_dev,
                        const double* state_old_dev, const double* Vu_dev, double* Kv_u_dev, void* stream);

/* Linear solve after assembly: conjugate gradients on the assembled CSC
 * stiffness over the unknowns (nzval from fec_assemble; symmetric), K x = b,
 * starting from x.  preconditioner 0: none (the reference's Krylov CG), 1:
 * Jacobi.  Stops at ||b - K x|| <= rtol ||b|| (checked every 10 iterations) or
 * after max_iter; reports the iterations and the final relative residual.
 * Bitwise repeatable.  Synchronises the stream.  Replaces the Krylov solve of
 * IterativeLinearSolver (src/Solvers.jl:88-152). */
int fec_cg_solve(fec_ctx* ctx, const double* nzval_dev, const double* b_dev, double* x_dev, int max_iter,
                 double rtol, int preconditioner, int* iterations, double* rel_residual, void* stream);

/* Checks assembled outputs (either may be NULL): FEC_ERR_DEVICE if an element
 * kernel gave up a bounded wait (the flag of fec_tensor_core_status, not
 * cleared here; the outputs are then not to be trusted), else FEC_ERR_NONFINITE
 * if they hold NaN/Inf, with the first offending index (residual first, then
 * nzval; -1 if none) and a message naming the array, else FEC_OK.
 * Synchronises the stream.  The boundary's output check; the reference does
 * not check. */
int fec_check_finite(fec_ctx* ctx, const double* R_u_dev, const double* nzval_dev, int64_t* first_bad,
                     void* stream);

/* Assembly that allocates no device memory.  No counterpart in the reference.
 *
 * fec_assemble keeps its element-matrix workspace in memory it cudaMallocs on
 * first use.  Callers that cannot let a library allocate -- applications whose
 * device memory all goes through their own pool (CUDA.jl's pool, PyTorch's
 * caching allocator), where a private cudaMalloc escapes the pool's accounting
 * and a cudaFree synchronizes the device mid-step, or callers with a device
 * memory budget fixed up front -- call this instead.  Same arguments, and the
 * same kernels as fec_assemble, so bitwise the same results, with one
 * exception: hex8 blocks of FEC_PHYS_J2_MLP in FEC_FP32_ELEMENT arithmetic
 * evaluate the learned closure per point on the CUDA cores here (the
 * tensor-core closure needs a per-point table the size of the mesh), which is
 * what fec_assemble does with FEC_CLOSURE_ON_CUDA_CORES=1; their outputs and
 * closure counters then differ from fec_assemble's tensor-core results within
 * the closure's own tolerance.  The context still has to be set up (mesh,
 * dofs, pattern) beforehand, and the inputs and outputs are the caller's.
 * No launch of this call is timed (fec_kernel_times reports none after it).
 *
 * Its workspace is one static device array of FEC_NOALLOC_SCRATCH_BYTES that
 * every GPU which loads the library holds until the process exits.  Meshes
 * whose element workspace (NE * NDOF^2 element-matrix entries -- the symmetric
 * half, NE * A(A+1)/2 * 9, for blocks of translated elements whose tensor-core
 * kernels write only that -- plus NE * NDOF element-residual entries, 8 bytes
 * each in FP64, 4 in FP32) exceeds it are rejected with FEC_ERR_ARG.  Every call made outside stream capture looks up
 * the array's device address (cudaGetSymbolAddress), so a reset of the
 * device's primary context in between is harmless; a call under capture uses
 * the address of the last call on that device, so make the first call on a
 * device (and the first after a reset) before any stream capture.  All calls
 * share the array: calls whose work overlaps on the GPU (different streams,
 * different contexts) race on it.  Nothing in it needs clearing, as every
 * element rewrites its entries before they are read. */
#define FEC_NOALLOC_SCRATCH_BYTES (64u << 20)
int fec_assemble_noalloc(fec_ctx* ctx, int want, int precision, double t, double dt, const double* U_dev,
                         const double* U_old_dev, const double* state_old_dev, double* state_new_dev,
                         double* R_u_dev, double* nzval_dev, void* stream);

/* Learned closure (no counterpart in the reference, whose physics are Julia
 * functions; the J2 return map it replaces is the project's own).  ------------ */

/* Number of MLP parameters (14-64-64-64-64-13, SiLU; per layer W [out][in]
 * row-major then b). */
int fec_mlp_param_count(void);
/* Exact J2 radial return of n points (FP64, device arrays): strain (6 tensor
 * components xx yy zz yz xz xy per point), state (7) -> stress (6), new state
 * (7), and optionally the 6x6 consistent tangent d sigma / d eps.  props as
 * FEC_PHYS_J2.  Used to generate training data and as the reference for the closure's error. */
int fec_j2_points(const double* props, int64_t n, const double* strain_dev, const double* state_old_dev,
                  double* stress_dev, double* state_new_dev, double* tangent_dev, void* stream);
/* MLP forward pass on n normalised samples X (n x 14) -> Y (n x 13), FP32. */
int fec_mlp_forward(const float* params_dev, const float* X_dev, int64_t n, float* Y_dev, void* stream);
/* Gradient of the mean squared error against targets Y, summed in a fixed
 * order; scratch needs ceil(n/64) * (params + 1) floats. */
int fec_mlp_gradient(const float* params_dev, const float* X_dev, const float* Y_dev, int64_t n, float* scratch_dev,
                     int64_t scratch_len, float* grad_dev, float* loss_dev, void* stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on the batch (X, Y); step >= 1. */
int fec_mlp_adam_step(float* params_dev, float* m_dev, float* v_dev, const float* X_dev, const float* Y_dev,
                      int64_t n, int64_t step, float lr, float* scratch_dev, int64_t scratch_len, float* loss_dev,
                      void* stream);
/* The network on the tensor cores, as the assembly runs it: n rows of X (device,
 * n x 14, physical units) -> outputs Y (n x 13, physical units) and the Jacobian
 * of the six stress outputs with respect to the six strain inputs (n x 36,
 * row-major 6 x 6).  Parameters and normalisation on the host, as for
 * fec_closure_set.  Synchronises the stream.  No counterpart in the reference. */
int fec_mlp_eval_tc(const float* params, const float* normalisation, const float* X_dev, int64_t n, float* Y_dev,
                    float* jac_dev, void* stream);
/* Installs a trained closure for FEC_PHYS_J2_MLP blocks: FP32 parameters (host;
 * the device keeps a BF16 copy and the two-term BF16 split the tensor-core
 * kernel uses), the feature normalisation (host; 14 + 14 + 13 + 13 floats:
 * input mean, input std, output mean, output std) and the consistency threshold
 * (relative to sigma_y) above which a point falls back to the exact update.
 * Hex8 blocks assembled with FEC_FP32_ELEMENT run the network on the tensor
 * cores; other combinations evaluate it per point on the CUDA cores. */
int fec_closure_set(fec_ctx* ctx, const float* params, const float* normalisation, float tol);
/* Plastic points that used the closure path and fallbacks since the last reset. */
int fec_closure_stats(fec_ctx* ctx, int64_t* plastic_points, int64_t* fallbacks, int reset);

/* Number of kernels fec_assemble launched in the last call (for accounting). */
int fec_last_launch_count(const fec_ctx* ctx);

/* Measurement helpers (no counterpart in the reference, which only times whole
 * sections with TimerOutputs, src/Solvers.jl:133-151). ------------------------ */

/* When on, fec_update_field/fec_assemble bracket each kernel launch with a CUDA
 * event pair on the caller's stream.  Off by default. */
int fec_set_profiling(fec_ctx* ctx, int on);
/* Durations (ms) of the launches timed by the last fec_update_field +
 * fec_assemble pair, in launch order; names gets a comma-separated list.
 * Waits for those events.  Returns the number of timed launches (>= 0). */
int fec_kernel_times(fec_ctx* ctx, float* ms, int cap, char* names, size_t len);
/* FMA throughput probe on `device` (TFLOP/s, 2 flops per FMA) in FP64
 * (precision FEC_FP64) or FP32 (FEC_FP32_ELEMENT): the denominator of the
 * FP64-bound roofline of the element kernels. */
int fec_probe_fma_rate(int device, int precision, double* tflops);
/* Self-check of the FP64 path's conversions (device buffers, stream-ordered):
 * for each x[i], split[2i], split[2i+1] = the double-float (hi, lo) the FP64
 * kernels form from it, and widened[2i], widened[2i+1] = hi and lo widened back
 * to double as the node gather does.  No reference counterpart. */
int fec_df64_split_check(const double* x_dev, int64_t n, float* split_dev, double* widened_dev, void* stream);

/* Sizes the context knows (any pointer may be NULL). */
/* Launch configurations the autotuner chose for the generic element kernels
 * (tet4/tet10/hex27: elements per CTA, threads per element), one text line per
 * tuned kernel family and problem-size bucket with every candidate's time.
 * Returns the number of lines.  Tuning happens on a family's first launch
 * outside CUDA-graph capture; FEC_AUTOTUNE=0 keeps the defaults.  No
 * counterpart in the reference. */
int fec_autotune_report(char* buf, size_t len);
/* FEC_OK, or FEC_ERR_DEVICE if an element kernel on the current device gave
 * up a bounded wait -- a tensor-core kernel (hex27 FP32-element) waiting for
 * its MMAs, or a hex8 kernel waiting for the bulk copy of its reference tables
 * and connectivity (it then falls back to plain loads) -- since the flag was
 * last cleared; the results of that call are then not to be trusted.  reset
 * clears the flag.  fec_check_finite reports the same flag.  Synchronous.  No
 * counterpart in the reference. */
int fec_tensor_core_status(int reset);
/* SM clocks the element kernels' bounded waits allow before they give up:
 * the main waits of the hex27 tensor-core kernel (hex27 FP32-element) and the
 * hex8 kernels' wait on their bulk table copy (FEC_HEX8_DF64=tile and the
 * FP32-element hex8 kernel).  0 (the default) is about one second.  The drain
 * that follows a timeout always allows the full second.  Process-wide; for
 * testing the timeout path on operations that complete anyway.  No
 * counterpart in the reference. */
int fec_set_wait_budget(long long clocks);
int fec_sizes(const fec_ctx* ctx, int64_t* num_nodes, int64_t* num_elems, int64_t* num_unknowns, int64_t* nnz,
              int64_t* state_len);

#ifdef __cplusplus
}
#endif
#endif /* FEC_GB300_H */
