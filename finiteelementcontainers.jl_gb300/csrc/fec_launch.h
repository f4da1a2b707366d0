// fec_launch.h -- host-side launchers of the kernels in fec_kernels.cuh.
// Each physics family is instantiated in its own translation unit so the
// library builds in parallel.
#pragma once
#include <vector>
#include <cuda_runtime.h>
#include "fec_kernels.cuh"

namespace fec {

// Raises a kernel's dynamic shared-memory limit once per device (and again only
// when a larger size is asked for), so that launches recorded during CUDA graph
// capture issue no attribute calls.  One instance per kernel.
template <auto Kern>
inline cudaError_t ensure_smem(size_t bytes) {
  static int set_bytes[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && int(bytes) <= set_bytes[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e == cudaSuccess && dev >= 0 && dev < 64) set_bytes[dev] = int(bytes);
  return e;
}

// Return cudaSuccess, or cudaErrorNotSupported for a combination that is not
// built.  *launches is incremented by the kernels launched.
cudaError_t launch_poisson(int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& args,
                           cudaStream_t stream, int* launches);
cudaError_t launch_mech(int physics, int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& args,
                        cudaStream_t stream, int* launches);
cudaError_t launch_gather(int precision, int nf, const GatherArgs& args, cudaStream_t stream, int* launches);
// The node gather of a mesh of mixed element sizes, one launch per group of nodes:
// nodes[off .. off + count) are the nodes whose adjacent elements all have A nodes
// (A = 4, 8, 10 or 27: the gather with that element size at compile time, several
// elements' loads in flight), A = 0 the rest (shared between element sizes).  The
// groups partition the nodes; the results are bitwise those of launch_gather.
struct NodeGroup {
  int A;
  int64_t off, count;
};
cudaError_t launch_gather_groups(int precision, int nf, const GatherArgs& args, const int32_t* nodes,
                                 const NodeGroup* groups, int ngroups, cudaStream_t stream, int* launches);
// Matrix-free tangent action: element contributions K_e v_e (summed over points
// in point order) into the residual workspace args.Re; V is the full direction
// field (zero on Dirichlet dofs).  The state is read only.
cudaError_t launch_action(int physics, int elem_type, int precision, const ElemArgs& args, const double* V,
                          cudaStream_t stream, int* launches);
// Hex27 FP32-element mechanics with the element-stiffness contraction on the
// tensor cores (physics 2 Neo-Hookean, 3 J2); a wait that gives up sets the
// flag fec_tensor_core_status reads.
// Device address of that flag on the current device (an int, nonzero once an
// element kernel's bounded wait gave up; ElemArgs::wait_err points at it).
cudaError_t wait_error_flag(int** flag);
cudaError_t launch_hex27_tc(int physics, bool want_r, bool want_k, const ElemArgs& args, cudaStream_t stream,
                            int* launches);
// FEC_HEX27_ON_CUDA_CORES=1 keeps hex27 FP32-element blocks on the generic kernel.
bool hex27_on_cuda_cores();
// FP64 Neo-Hookean (2) or J2 (3) element blocks of types hex8/tet4/tet10/hex27
// (at most MIXED_MAX_BLOCKS) in one persistent launch; bitwise the per-block result.
// tile_counter: one unsigned of device memory, zeroed on `stream` by the launch
// (the CTAs take their work tiles from it).
constexpr int MIXED_MAX_BLOCKS = 4;
bool mixed_launch_supported(int physics, int nblocks, const int* elem_types);
cudaError_t launch_mech_mixed(int physics, int nblocks, const int* elem_types, const ElemArgs* args, bool want_r,
                              bool want_k, unsigned* tile_counter, cudaStream_t stream, int* launches);

// Streaming multiprocessors of the current device (cached per device).
int num_sms();
// FP64 hex8 Neo-Hookean (2) or J2 (3) for a block whose elements are
// translates of its first one (args.affine: the table hex8_affine_table built):
// with the tangent, its contraction on the tensor cores in exact 8-bit digit
// slices; residual-only calls run the same point phase and residual arithmetic.
cudaError_t launch_hex8_affine_tc(int physics, bool want_r, bool want_k, const ElemArgs& args, cudaStream_t stream,
                                  int* launches);
// Host: that table from the first element's node coordinates x0[8][3] and the
// block's reference tables (RefLayout<1>); false for a degenerate element.
bool hex8_affine_table(const double* x0, const double* ref, std::vector<unsigned char>& out);
// FEC_HEX8_AFFINE=0 keeps such blocks on the per-element kernels.
bool hex8_affine_enabled();
// Byte offset, in that table, of the block's spatial gradients dNX [8 points][8
// nodes][3] (double), followed by JxW [8] (double): the same for every element.
size_t hex8_affine_grad_offset();
// With the stiffness that kernel writes the symmetric half of K_e (args.ke_pairs:
// the KE_PAIRS layout, 36 * 9 entries per element) unless FEC_HEX8_PAIRS=0
// (the node rows of the whole K_e, KE_NODE_ROWS).
bool hex8_pairs_enabled();
// Tet10 (7) / hex27 (8) Neo-Hookean (2) or J2 (3) for a block whose element e is
// a translate of element e mod P (args.affine: the table class_tc_table built):
// the stiffness contraction on the tensor cores against each class's constant
// gradient products -- FP32-element (precision 1, tet10 and hex27) with
// kind::tf32 two-term splits, FP64 (precision 0, tet10) with exact BF16 digit
// slices; residual-only calls run the same point phase and residual arithmetic.
cudaError_t launch_class_tc(int physics, int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& args,
                            cudaStream_t stream, int* launches);
// Host: that table for nclass (<= 8) classes from the classes' first elements'
// node coordinates xc[nclass][A][3] and the block's reference tables
// (RefLayout order); false for an inverted or degenerate element.
bool class_tc_table(int elem_type, int nclass, const double* xc, const double* ref, std::vector<unsigned char>& out);
// FEC_CLASS_TC=0 keeps such blocks on the per-element kernels.
bool class_tc_enabled();
// Whether an assembly of such a block (physics, element type, precision, residual
// and stiffness wanted, a class table present) runs that kernel; with the
// stiffness it writes the KE_PAIRS workspace layout (A(A+1)/2 * 9 entries per
// element).
bool class_tc_runs(int physics, int elem_type, int precision, bool want_r, bool want_k, bool has_table);
// FEC_HEX8_DF64=tile selects the one-tile-per-CTA FP64 hex8 kernel instead of
// the warp-specialised persistent one.
bool hex8_df64_tile_kernel();

// Reference-element tables (RefLayout order) for an element type, in double.
// Returns the number of doubles written (0 for an unknown type).
int ref_tables(int elem_type, double* out, int cap);
int elem_nnpe(int elem_type);
int elem_dim(int elem_type);
int elem_nq(int elem_type);

}  // namespace fec
