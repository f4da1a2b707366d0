// fec_abi.cu -- the C ABI of libfec_gb300.so (declared in include/fec_gb300.h):
// context, mesh/physics/DOF set-up, the symbolic phase that builds the CSC
// pattern and the element -> nzval maps, and the assembly driver.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/fec_gb300.h"
#include "fec_closure.cuh"
#include "fec_closure_tc.h"
#include "fec_launch.h"
#include "fec_pattern.h"
#include "fec_solver.h"
#include <cuda_bf16.h>

using fec::BlockInfo;
using fec::ElemArgs;
using fec::GatherArgs;

namespace {

thread_local int g_create_status = FEC_OK;
// SM clocks the element kernels' bounded waits allow (0: their default, about 1 s)
long long g_wait_budget = 0;
thread_local char g_create_msg[256] = "";

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

struct Block {
  int elem_type = 0, nnpe = 0, nq = 0;
  int64_t ne = 0;
  int64_t elem_start = 0, conn_off = 0, epos_off = 0;
  int physics = 0;
  double props[8] = {0};
  int nprops = 0;
  // hex8 block whose elements are translates of the first one (node offsets
  // within 1e-13 of the element size): x0 = the first element's coordinates
  bool congruent = false;
  double x0[24] = {0};
  // tet10/hex27 block whose element e is a translate of element e mod nclass
  // (nclass <= 8, 0: none): xc = the first nclass elements' node coordinates
  int nclass = 0;
  std::vector<double> xc;
};

}  // namespace

struct fec_ctx {
  int device = 0;
  int status = FEC_OK;
  std::string msg;
  int last_launches = 0;
  // mesh
  int dim = 0;
  int64_t nn = 0, ne_total = 0;
  std::vector<Block> blocks;
  std::vector<int32_t> conn;  // 0-based, all blocks
  // dofs
  int nf = 0;
  int64_t n_unknowns = -1;
  std::vector<int64_t> dof_to_unknown;  // 0-based index or -1
  std::vector<uint8_t> umask;
  // pattern
  bool pattern_ready = false;
  int64_t nnz = 0;
  std::vector<int64_t> nbr_ptr;
  std::vector<int32_t> nbr;
  std::vector<int64_t> col_base;
  std::vector<int32_t> col_len;
  int acc_stride = 0;
  // device
  DevBuf d_coords, d_conn, d_ref, d_nadj_ptr, d_nadj, d_epos, d_umask, d_col_base, d_col_len, d_dtu, d_unknown_dofs;
  DevBuf d_Ke, d_Re;
  std::vector<int64_t> ref_off;  // per block offset (doubles) into d_ref
  std::vector<double> ref_host;  // host copy of d_ref (all blocks' tables)
  // learned closure (FEC_PHYS_J2_MLP): BF16 parameters, normalisation, counters, and the
  // ClosureArgs struct the kernels read
  DevBuf d_cl_w, d_cl_norm, d_cl_cnt, d_cl_args;
  DevBuf d_cl_img, d_cl_table;  // tensor-core closure: packed parameters, per-point table
  DevBuf d_V;                   // matrix-free action: the direction as a full field
  DevBuf d_colptr0, d_rowval32, d_cg;  // linear solve: 0-based CSC pattern, CG scratch
  DevBuf d_flag;                       // non-finite scan result
  DevBuf d_nbr_ptr, d_nbr;             // neighbour lists on the device (device symbolic phase, CSC fill)
  DevBuf d_tile_counter;               // single launch of mixed element blocks: next work tile
  // node gather of a mesh of mixed element sizes: the nodes grouped by the element
  // size of their adjacent elements (built on first use, per pattern)
  DevBuf d_node_groups;
  std::vector<fec::NodeGroup> node_groups;
  bool groups_ready = false;
  std::vector<DevBuf> d_affine;        // per block: the tensor-core operand table of a congruent hex8 block
                                       // or of a tet10/hex27 block of translation classes
  bool single_launch = false;          // FP64 mechanics: every element block in one launch
  float cl_tol = 0.f;
  // optional per-launch timing (CUDA events on the caller's stream)
  bool profiling = false;
  std::vector<cudaEvent_t> events;  // 2 per timed launch
  std::vector<std::string> ev_names;
  int n_timed = 0;
};

namespace {

int fail(fec_ctx* c, int status, const char* fmt, ...) {
  char buf[240];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) {
    c->status = status;
    c->msg = buf;
  } else {
    g_create_status = status;
    snprintf(g_create_msg, sizeof g_create_msg, "%s", buf);
  }
  return status;
}

int ok(fec_ctx* c) {
  c->status = FEC_OK;
  c->msg.clear();
  return FEC_OK;
}

#define FEC_CUDA(ctx, call)                                                                             \
  do {                                                                                                  \
    cudaError_t _e = (call);                                                                            \
    if (_e != cudaSuccess) return fail(ctx, FEC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_e));    \
  } while (0)

// FEC_FP64_CONTRACTION=native keeps the FP64 mechanics on the all-FP64 kernels
// (per block).
bool fp64_native_env() {
  static const bool v = [] {
    const char* e = std::getenv("FEC_FP64_CONTRACTION");
    return e && e[0] == 'n';
  }();
  return v;
}

int upload(fec_ctx* c, DevBuf& b, const void* src, size_t bytes) {
  b.release();
  if (bytes == 0 || c->device < 0) return FEC_OK;
  FEC_CUDA(c, cudaMalloc(&b.p, bytes));
  b.bytes = bytes;
  FEC_CUDA(c, cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice));
  return FEC_OK;
}

// The tensor-core operand table of block b (hex8, elements translates of the
// first), from its current reference tables; none for other blocks, on a
// host-only context, or for a degenerate first element.
int build_affine(fec_ctx* c, size_t b) {
  if (c->d_affine.size() != c->blocks.size()) c->d_affine.resize(c->blocks.size());
  DevBuf& d = c->d_affine[b];
  d.release();
  const Block& B = c->blocks[b];
  if (c->device < 0) return FEC_OK;
  std::vector<unsigned char> tab;
  if (B.congruent) {
    if (!fec::hex8_affine_table(B.x0, c->ref_host.data() + c->ref_off[b], tab)) return FEC_OK;
  } else if (B.nclass > 0) {
    if (!fec::class_tc_table(B.elem_type, B.nclass, B.xc.data(), c->ref_host.data() + c->ref_off[b], tab))
      return FEC_OK;
  } else {
    return FEC_OK;
  }
  return upload(c, d, tab.data(), tab.size());
}

// The table a launch of block b may use: FP64 assemblies of congruent hex8
// blocks on their own launch (the single launch across blocks keeps the
// per-element kernels), unless FEC_HEX8_AFFINE=0.
// Assemblies of tet10/hex27 blocks of translation classes get theirs: FP32-element
// and FP64 (tet10: the tensor-core kernels; hex27 FP64: the class gradients).
const void* affine_table(const fec_ctx* c, size_t b, int precision, bool mixed) {
  if (mixed || b >= c->d_affine.size()) return nullptr;
  if (c->blocks[b].elem_type == FEC_HEX8)
    return precision == FEC_FP64 && fec::hex8_affine_enabled() ? c->d_affine[b].p : nullptr;
  return (precision == FEC_FP32_ELEMENT || precision == FEC_FP64) ? c->d_affine[b].p : nullptr;
}

int ensure(fec_ctx* c, DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes) return FEC_OK;
  b.release();
  FEC_CUDA(c, cudaMalloc(&b.p, bytes));
  b.bytes = bytes;
  return FEC_OK;
}

// element-matrix blocks start on 16-byte boundaries (vectorised copy-out)
inline int64_t pad4(int64_t n) { return (n + 3) & ~int64_t(3); }

// FEC_HEX27_PAIRS=0: the FP64 hex27 double-float kernel writes its element
// matrices whole (row-major) instead of the symmetric half; the same values.
bool hex27_pairs_enabled() {
  const char* v = std::getenv("FEC_HEX27_PAIRS");
  return !(v && v[0] == '0');
}

// Whether an assembly of block b with the stiffness runs an FP64 element kernel
// that writes the symmetric half of K_e (KE_PAIRS): the hex8 tensor-core kernel
// (instead of node rows, unless FEC_HEX8_PAIRS=0) and the hex27 double-float
// kernel (on its own launch, unless FEC_HEX27_PAIRS=0).
bool fp64_pairs(const fec_ctx* c, size_t b, int precision, bool want_k, bool mixed) {
  const Block& B = c->blocks[b];
  if (!want_k || precision != FEC_FP64 || fp64_native_env() ||
      !(B.physics == FEC_PHYS_NEOHOOKEAN || B.physics == FEC_PHYS_J2))
    return false;
  if (B.elem_type == FEC_HEX27) return !mixed && hex27_pairs_enabled();
  return B.elem_type == FEC_HEX8 && fec::hex8_pairs_enabled() && affine_table(c, b, precision, mixed) != nullptr;
}

// Workspace entries of block b's element matrices: the class tensor-core kernels
// and the FP64 hex8 tensor-core kernel write the symmetric half (KE_PAIRS), every
// other kernel the whole K_e.  `mixed`: the single launch across blocks.
int64_t ke_entries(const fec_ctx* c, size_t b, int precision, bool want_k, bool mixed) {
  const Block& B = c->blocks[b];
  if (fp64_pairs(c, b, precision, want_k, mixed) ||
      (want_k && fec::class_tc_runs(B.physics, B.elem_type, precision, true, want_k,
                                    affine_table(c, b, precision, mixed) != nullptr)))
    return pad4(B.ne * (int64_t(B.nnpe) * (B.nnpe + 1) / 2 * 9));
  const int ndof = c->nf * B.nnpe;
  return pad4(B.ne * ndof * ndof);
}

// FEC_CLOSURE_ON_CUDA_CORES=1 selects the per-thread network evaluation (the
// generic element kernel) instead of the tensor-core closure kernel.
bool closure_on_cuda_cores() {
  const char* v = std::getenv("FEC_CLOSURE_ON_CUDA_CORES");
  return v && v[0] == '1';
}

// Learned-closure hex8 blocks in FP32 element arithmetic run the tensor-core
// closure kernel and the FP32 hex8 element kernel (node-rows layout).
bool tc_closure(const Block& B, int precision) {
  return B.physics == FEC_PHYS_J2_MLP && B.elem_type == FEC_HEX8 && precision == FEC_FP32_ELEMENT &&
         !closure_on_cuda_cores();
}

int num_fields_of(int physics) { return physics == FEC_PHYS_POISSON ? 1 : 3; }
int num_states_of(int physics) { return (physics == FEC_PHYS_J2 || physics == FEC_PHYS_J2_MLP) ? 7 : 0; }

// U[bc_dofs[i]-1] = vals[i]
__global__ void set_dirichlet_kernel(double* U, int64_t n, const int64_t* dofs, const double* vals) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) U[dofs[i] - 1] = vals[i];
}

// U[unknown_dofs[k]] = Uu[k]  (unknown_dofs 0-based here)
__global__ void set_unknowns_kernel(double* U, int64_t n, const int64_t* unknown_dofs, const double* Uu) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < n) U[unknown_dofs[k]] = Uu[k];
}

// Smallest index of a non-finite entry of x[0..n) into *first (atomicMin).
__global__ void first_nonfinite_kernel(const double* x, int64_t n, unsigned long long* first) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    if (!isfinite(x[i])) atomicMin(first, (unsigned long long)i);
}

// Records an event pair around launch `name` when profiling is on.
struct LaunchTimer {
  fec_ctx* c;
  cudaStream_t s;
  int slot = -1;
  LaunchTimer(fec_ctx* c_, cudaStream_t s_, const char* name) : c(c_), s(s_) {
    if (!c->profiling) return;
    slot = c->n_timed;
    if (int(c->events.size()) < 2 * (slot + 1)) {
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess) { slot = -1; return; }
      if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); slot = -1; return; }
      c->events.push_back(a);
      c->events.push_back(b);
    }
    if (int(c->ev_names.size()) <= slot) c->ev_names.resize(slot + 1);
    c->ev_names[slot] = name;
    cudaEventRecord(c->events[2 * slot], s);
  }
  ~LaunchTimer() {
    if (slot < 0) return;
    cudaEventRecord(c->events[2 * slot + 1], s);
    c->n_timed = slot + 1;
  }
};

// FEC_GATHER_RUNS=generic gathers a mesh of mixed element sizes in one launch on
// the one-element-at-a-time routine (bitwise the same results as the groups).
bool gather_runs_generic() {
  const char* e = getenv("FEC_GATHER_RUNS");
  return e && e[0] == 'g';
}

// The node groups of launch_gather_groups: a node whose adjacent elements all come
// from one block joins the group of that block's element size (4, 8, 10, 27), every
// other node (elements of several blocks, or none) the group A = 0.
int build_node_groups(fec_ctx* c) {
  std::vector<int> owner(size_t(c->nn), -1);
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    for (int64_t i = 0; i < B.ne * B.nnpe; ++i) {
      int& o = owner[size_t(c->conn[B.conn_off + i])];
      o = (o == -1 || o == int(b)) ? int(b) : -2;
    }
  }
  static const int kSizes[5] = {4, 8, 10, 27, 0};
  std::vector<int32_t> list;
  list.reserve(size_t(c->nn));
  c->node_groups.clear();
  for (int gi = 0; gi < 5; ++gi) {
    const int64_t off = int64_t(list.size());
    for (int64_t n = 0; n < c->nn; ++n) {
      const int A = owner[size_t(n)] >= 0 ? c->blocks[size_t(owner[size_t(n)])].nnpe : 0;
      const int Ag = (A == 4 || A == 8 || A == 10 || A == 27) ? A : 0;
      if (Ag == kSizes[gi]) list.push_back(int32_t(n));
    }
    if (int64_t(list.size()) > off) c->node_groups.push_back({kSizes[gi], off, int64_t(list.size()) - off});
  }
  if (int rc = upload(c, c->d_node_groups, list.data(), sizeof(int32_t) * list.size())) return rc;
  c->groups_ready = true;
  return FEC_OK;
}

void invalidate_pattern(fec_ctx* c) {
  c->pattern_ready = false;
  c->groups_ready = false;
  c->d_node_groups.release();
  c->nnz = 0;
  c->d_colptr0.release();
  c->d_rowval32.release();
  c->d_nadj_ptr.release();
  c->d_nadj.release();
  c->d_epos.release();
  c->d_col_base.release();
  c->d_col_len.release();
  c->d_nbr_ptr.release();
  c->d_nbr.release();
}

}  // namespace

extern "C" {

int fec_ctx_create(int device, fec_ctx** out) {
  if (!out) return fail(nullptr, FEC_ERR_ARG, "fec_ctx_create: out is NULL");
  *out = nullptr;
  if (device == -1) {  // host-only context: mesh, dofs and the symbolic phase
    fec_ctx* c = new fec_ctx();
    c->device = -1;
    *out = c;
    g_create_status = FEC_OK;
    g_create_msg[0] = 0;
    return FEC_OK;
  }
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) return fail(nullptr, FEC_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
  if (device < 0 || device >= count) return fail(nullptr, FEC_ERR_ARG, "device %d out of range (%d)", device, count);
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(nullptr, FEC_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  fec_ctx* c = new fec_ctx();
  c->device = device;
  *out = c;
  g_create_status = FEC_OK;
  g_create_msg[0] = 0;
  return FEC_OK;
}

int fec_ctx_destroy(fec_ctx* c) {
  if (!c) return FEC_OK;
  if (c->device >= 0) cudaSetDevice(c->device);
  for (cudaEvent_t e : c->events) cudaEventDestroy(e);
  for (DevBuf* b : {&c->d_coords, &c->d_conn, &c->d_ref, &c->d_nadj_ptr, &c->d_nadj, &c->d_epos, &c->d_umask,
                    &c->d_col_base, &c->d_col_len, &c->d_dtu, &c->d_unknown_dofs, &c->d_Ke, &c->d_Re, &c->d_cl_w,
                    &c->d_cl_norm, &c->d_cl_cnt, &c->d_cl_args, &c->d_cl_img, &c->d_cl_table, &c->d_V, &c->d_colptr0, &c->d_rowval32,
                    &c->d_cg, &c->d_flag, &c->d_nbr_ptr, &c->d_nbr, &c->d_tile_counter, &c->d_node_groups})
    b->release();
  for (DevBuf& b : c->d_affine) b.release();
  delete c;
  return FEC_OK;
}

int fec_last_error(const fec_ctx* c, char* buf, size_t len) {
  const char* m = c ? c->msg.c_str() : g_create_msg;
  if (buf && len) {
    strncpy(buf, m, len - 1);
    buf[len - 1] = 0;
  }
  return c ? c->status : g_create_status;
}

int fec_last_launch_count(const fec_ctx* c) { return c ? c->last_launches : 0; }

int fec_sizes(const fec_ctx* c, int64_t* nn, int64_t* ne, int64_t* nu, int64_t* nnz, int64_t* state_len) {
  if (!c) return FEC_ERR_ARG;
  if (nn) *nn = c->nn;
  if (ne) *ne = c->ne_total;
  if (nu) *nu = c->n_unknowns;
  if (nnz) *nnz = c->nnz;
  if (state_len) {
    int64_t s = 0;
    for (const Block& b : c->blocks) s += int64_t(num_states_of(b.physics)) * b.nq * b.ne;
    *state_len = s;
  }
  return FEC_OK;
}

int fec_mesh_set(fec_ctx* c, int dim, int64_t nn, const double* coords, int nblocks, const int32_t* elem_types,
                 const int64_t* block_ne, const int64_t* conn) {
  if (!c) return FEC_ERR_ARG;
  if (dim != 2 && dim != 3) return fail(c, FEC_ERR_ARG, "dim must be 2 or 3 (got %d)", dim);
  if (nn <= 0 || !coords) return fail(c, FEC_ERR_ARG, "need num_nodes > 0 and coords");
  if (nblocks <= 0 || nblocks > fec::MAX_BLOCKS)
    return fail(c, FEC_ERR_ARG, "num_blocks must be in 1..%d (got %d)", fec::MAX_BLOCKS, nblocks);
  if (nn >= (int64_t(1) << 31)) return fail(c, FEC_ERR_ARG, "num_nodes must be < 2^31");
  if (c->device >= 0) cudaSetDevice(c->device);
  std::vector<Block> blocks(nblocks);
  int64_t total_conn = 0, ne_total = 0, epos_total = 0;
  for (int b = 0; b < nblocks; ++b) {
    Block& B = blocks[b];
    B.elem_type = elem_types[b];
    B.nnpe = fec::elem_nnpe(B.elem_type);
    B.nq = fec::elem_nq(B.elem_type);
    if (!B.nnpe) return fail(c, FEC_ERR_UNSUPPORTED, "block %d: unsupported element type %d", b + 1, B.elem_type);
    if (fec::elem_dim(B.elem_type) != dim)
      return fail(c, FEC_ERR_ARG, "block %d: element type %d is not %dD", b + 1, B.elem_type, dim);
    if (block_ne[b] < 0) return fail(c, FEC_ERR_ARG, "block %d: negative element count", b + 1);
    B.ne = block_ne[b];
    B.elem_start = ne_total;
    B.conn_off = total_conn;
    B.epos_off = epos_total;
    ne_total += B.ne;
    total_conn += B.ne * B.nnpe;
    epos_total += (B.ne * B.nnpe * B.nnpe + 3) & ~int64_t(3);  // 8-byte aligned blocks
  }
  if (ne_total >= (int64_t(1) << 58)) return fail(c, FEC_ERR_ARG, "too many elements");
  std::vector<int32_t> conn0(total_conn);
  int64_t bad = -1;
#pragma omp parallel for schedule(static) reduction(max : bad)
  for (int64_t i = 0; i < total_conn; ++i) {
    const int64_t v = conn[i];
    if (v < 1 || v > nn) bad = std::max(bad, i);
    conn0[i] = int32_t(v - 1);
  }
  if (bad >= 0)
    return fail(c, FEC_ERR_ARG, "connectivity entry %lld = %lld is outside 1..%lld", (long long)bad + 1,
                (long long)conn[bad], (long long)nn);
  // elements must not repeat a node (the gather relies on distinct slots)
  for (const Block& B : blocks) {
    int64_t dup = -1;
#pragma omp parallel for schedule(static) reduction(max : dup)
    for (int64_t e = 0; e < B.ne; ++e) {
      const int32_t* ce = conn0.data() + B.conn_off + e * B.nnpe;
      for (int a = 0; a < B.nnpe; ++a)
        for (int b2 = a + 1; b2 < B.nnpe; ++b2)
          if (ce[a] == ce[b2]) dup = std::max(dup, e);
    }
    if (dup >= 0) return fail(c, FEC_ERR_ARG, "element %lld repeats a node", (long long)(B.elem_start + dup + 1));
  }
  // hex8 blocks whose elements are all translates of the first one
  for (Block& B : blocks) {
    if (B.elem_type != 1 || dim != 3 || B.ne < 1) continue;
    const int32_t* c0 = conn0.data() + B.conn_off;
    double d0[24], h = 0.0;
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d) {
        B.x0[a * 3 + d] = coords[int64_t(c0[a]) * 3 + d];
        d0[a * 3 + d] = coords[int64_t(c0[a]) * 3 + d] - coords[int64_t(c0[0]) * 3 + d];
        h = std::max(h, std::fabs(d0[a * 3 + d]));
      }
    double dev = 0.0;
#pragma omp parallel for schedule(static) reduction(max : dev)
    for (int64_t e = 0; e < B.ne; ++e) {
      const int32_t* ce = conn0.data() + B.conn_off + e * 8;
      for (int a = 1; a < 8; ++a)
        for (int d = 0; d < 3; ++d) {
          const double off = coords[int64_t(ce[a]) * 3 + d] - coords[int64_t(ce[0]) * 3 + d];
          dev = std::max(dev, std::fabs(off - d0[a * 3 + d]));
        }
    }
    B.congruent = h > 0.0 && dev <= 1e-13 * h;
  }
  // tet10/hex27 blocks of translation classes: the smallest period P <= 8 such that
  // every element's node offsets X_e[a] - X_e[0] match element (e mod P)'s to within
  // 1e-13 of that element's size
  for (Block& B : blocks) {
    if ((B.elem_type != 7 && B.elem_type != 8) || dim != 3 || B.ne < 1) continue;
    const int A = B.nnpe;
    for (int P = 1; P <= 8 && P <= B.ne; ++P) {
      std::vector<double> d0(size_t(P) * A * 3), hc(P, 0.0);
      for (int cl = 0; cl < P; ++cl) {
        const int32_t* ce = conn0.data() + B.conn_off + int64_t(cl) * A;
        for (int a = 0; a < A; ++a)
          for (int d = 0; d < 3; ++d) {
            const double off = coords[int64_t(ce[a]) * 3 + d] - coords[int64_t(ce[0]) * 3 + d];
            d0[(size_t(cl) * A + a) * 3 + d] = off;
            hc[cl] = std::max(hc[cl], std::fabs(off));
          }
      }
      int bad = 0;  // (a bitwise-or reduction: each thread's copy starts at 0)
#pragma omp parallel for schedule(static) reduction(| : bad)
      for (int64_t e = 0; e < B.ne; ++e) {
        if (bad) continue;
        const int cl = int(e % P);
        const int32_t* ce = conn0.data() + B.conn_off + e * A;
        for (int a = 1; a < A && !bad; ++a)
          for (int d = 0; d < 3; ++d) {
            const double off = coords[int64_t(ce[a]) * 3 + d] - coords[int64_t(ce[0]) * 3 + d];
            if (!(std::fabs(off - d0[(size_t(cl) * A + a) * 3 + d]) <= 1e-13 * hc[cl])) bad = 1;
          }
      }
      if (bad) continue;
      B.nclass = P;
      B.xc.resize(size_t(P) * A * 3);
      for (int cl = 0; cl < P; ++cl) {
        const int32_t* ce = conn0.data() + B.conn_off + int64_t(cl) * A;
        for (int a = 0; a < A; ++a)
          for (int d = 0; d < 3; ++d) B.xc[(size_t(cl) * A + a) * 3 + d] = coords[int64_t(ce[a]) * 3 + d];
      }
      break;
    }
  }
  // reference tables
  std::vector<double> ref;
  std::vector<int64_t> ref_off(nblocks);
  for (int b = 0; b < nblocks; ++b) {
    double tmp[8192];
    const int n = fec::ref_tables(blocks[b].elem_type, tmp, 8192);
    ref_off[b] = int64_t(ref.size());
    ref.insert(ref.end(), tmp, tmp + n);
    while (ref.size() % 2) ref.push_back(0.0);
  }
  int rc;
  if ((rc = upload(c, c->d_coords, coords, sizeof(double) * size_t(nn) * dim))) return rc;
  if ((rc = upload(c, c->d_conn, conn0.data(), sizeof(int32_t) * conn0.size()))) return rc;
  if ((rc = upload(c, c->d_ref, ref.data(), sizeof(double) * ref.size()))) return rc;
  c->dim = dim;
  c->nn = nn;
  c->ne_total = ne_total;
  c->blocks = std::move(blocks);
  c->conn = std::move(conn0);
  c->ref_off = std::move(ref_off);
  c->ref_host = std::move(ref);
  for (DevBuf& d : c->d_affine) d.release();
  c->d_affine.assign(c->blocks.size(), DevBuf());
  for (size_t b = 0; b < c->blocks.size(); ++b)
    if ((rc = build_affine(c, b))) return rc;
  c->n_unknowns = -1;
  c->nf = 0;
  invalidate_pattern(c);
  return ok(c);
}

int fec_block_reference_set(fec_ctx* c, int block, int num_q, const double* N, const double* dN, const double* w) {
  if (!c) return FEC_ERR_ARG;
  if (block < 1 || block > int(c->blocks.size()))
    return fail(c, FEC_ERR_ARG, "block %d out of range 1..%d", block, int(c->blocks.size()));
  const Block& B = c->blocks[block - 1];
  const int A = B.nnpe, D = fec::elem_dim(B.elem_type), NQ = fec::elem_nq(B.elem_type);
  if (num_q != NQ)
    return fail(c, FEC_ERR_UNSUPPORTED,
                "block %d: the kernels of element type %d are built for %d quadrature points (got %d)", block,
                B.elem_type, NQ, num_q);
  if (!N || !dN || !w) return fail(c, FEC_ERR_ARG, "block %d: N, dN and w must not be NULL", block);
  // RefLayout order: N [q][a], dN [q][a][k], w [q]
  std::vector<double> t(size_t(NQ) * A * (1 + D) + NQ);
  std::copy(N, N + size_t(NQ) * A, t.begin());
  std::copy(dN, dN + size_t(NQ) * A * D, t.begin() + size_t(NQ) * A);
  std::copy(w, w + NQ, t.begin() + size_t(NQ) * A * (1 + D));
  for (size_t i = 0; i < t.size(); ++i)
    if (!std::isfinite(t[i])) return fail(c, FEC_ERR_ARG, "block %d: table entry %zu is not finite", block, i);
  std::copy(t.begin(), t.end(), c->ref_host.begin() + c->ref_off[block - 1]);
  if (c->device >= 0) {
    cudaSetDevice(c->device);
    // other blocks share the buffer: rewrite only this block's slice (kernels read it in stream order,
    // so the caller must not change tables while an assembly that uses them is in flight)
    FEC_CUDA(c, cudaMemcpy(static_cast<double*>(c->d_ref.p) + c->ref_off[block - 1], t.data(),
                           sizeof(double) * t.size(), cudaMemcpyHostToDevice));
  }
  int rc;
  if ((rc = build_affine(c, size_t(block - 1)))) return rc;
  return ok(c);
}

int fec_block_reference_get(const fec_ctx* cc, int block, int* num_q, double* N, double* dN, double* w) {
  fec_ctx* c = const_cast<fec_ctx*>(cc);
  if (!c) return FEC_ERR_ARG;
  if (block < 1 || block > int(c->blocks.size()))
    return fail(c, FEC_ERR_ARG, "block %d out of range 1..%d", block, int(c->blocks.size()));
  const Block& B = c->blocks[block - 1];
  const int A = B.nnpe, D = fec::elem_dim(B.elem_type), NQ = fec::elem_nq(B.elem_type);
  if (num_q) *num_q = NQ;
  const double* t = c->ref_host.data() + c->ref_off[block - 1];
  if (N) std::copy(t, t + size_t(NQ) * A, N);
  if (dN) std::copy(t + size_t(NQ) * A, t + size_t(NQ) * A * (1 + D), dN);
  if (w) std::copy(t + size_t(NQ) * A * (1 + D), t + size_t(NQ) * A * (1 + D) + NQ, w);
  return ok(c);
}

int fec_physics_set(fec_ctx* c, int block, int physics, const double* props, int nprops) {
  if (!c) return FEC_ERR_ARG;
  if (block < 1 || block > int(c->blocks.size()))
    return fail(c, FEC_ERR_ARG, "block %d out of range 1..%d", block, int(c->blocks.size()));
  if (physics != FEC_PHYS_POISSON && physics != FEC_PHYS_NEOHOOKEAN && physics != FEC_PHYS_J2 &&
      physics != FEC_PHYS_J2_MLP)
    return fail(c, FEC_ERR_UNSUPPORTED, "unknown physics %d", physics);
  const int need = physics == FEC_PHYS_POISSON ? 1 : (physics == FEC_PHYS_NEOHOOKEAN ? 2 : 4);
  if (nprops < need || nprops > 8 || (nprops > 0 && !props))
    return fail(c, FEC_ERR_ARG, "physics %d needs %d properties (got %d)", physics, need, nprops);
  Block& B = c->blocks[block - 1];
  if (physics != FEC_PHYS_POISSON && c->dim != 3)
    return fail(c, FEC_ERR_UNSUPPORTED, "mechanics physics needs a 3D mesh");
  B.physics = physics;
  B.nprops = nprops;
  for (int i = 0; i < 8; ++i) B.props[i] = i < nprops ? props[i] : 0.0;
  if (physics == FEC_PHYS_J2 || physics == FEC_PHYS_J2_MLP) fec::J2::fill_derived(B.props);  // slots 4-7
  return ok(c);
}

int fec_dofs_set(fec_ctx* c, int nf, const int64_t* dtu, int64_t n_unknowns) {
  if (!c) return FEC_ERR_ARG;
  if (c->nn <= 0) return fail(c, FEC_ERR_STATE, "fec_dofs_set before fec_mesh_set");
  if (nf != 1 && nf != 3) return fail(c, FEC_ERR_UNSUPPORTED, "num_fields must be 1 or 3 (got %d)", nf);
  if (!dtu) return fail(c, FEC_ERR_ARG, "dof_to_unknown is NULL");
  const int64_t ndofs = int64_t(nf) * c->nn;
  std::vector<int64_t> d(ndofs);
  std::vector<int64_t> unknown_dofs;
  unknown_dofs.reserve(size_t(std::max<int64_t>(n_unknowns, 0)));
  std::vector<uint8_t> um(c->nn, 0);
  int64_t next = 1;
  for (int64_t i = 0; i < ndofs; ++i) {
    const int64_t v = dtu[i];
    if (v == -1) {
      d[i] = -1;
      continue;
    }
    if (v != next)
      return fail(c, FEC_ERR_ARG,
                  "dof_to_unknown[%lld] = %lld: unknowns must be numbered 1..n in increasing dof order "
                  "(expected %lld or -1)",
                  (long long)i + 1, (long long)v, (long long)next);
    d[i] = v - 1;
    unknown_dofs.push_back(i);
    um[i / nf] |= uint8_t(1u << (i % nf));
    ++next;
  }
  if (next - 1 != n_unknowns)
    return fail(c, FEC_ERR_ARG, "num_unknowns = %lld but dof_to_unknown numbers %lld unknowns", (long long)n_unknowns,
                (long long)(next - 1));
  int rc;
  if ((rc = upload(c, c->d_dtu, d.data(), sizeof(int64_t) * d.size()))) return rc;
  if ((rc = upload(c, c->d_umask, um.data(), um.size()))) return rc;
  if ((rc = upload(c, c->d_unknown_dofs, unknown_dofs.data(), sizeof(int64_t) * unknown_dofs.size()))) return rc;
  c->nf = nf;
  c->n_unknowns = n_unknowns;
  c->dof_to_unknown = std::move(d);
  c->umask = std::move(um);
  invalidate_pattern(c);
  return ok(c);
}

int fec_pattern_build(fec_ctx* c, int64_t* nnz_out) {
  if (!c) return FEC_ERR_ARG;
  if (c->n_unknowns < 0) return fail(c, FEC_ERR_STATE, "fec_pattern_build before fec_dofs_set");
  if (c->device >= 0) cudaSetDevice(c->device);
  c->d_nbr_ptr.release();  // device copies of the neighbour lists go with the pattern
  c->d_nbr.release();
  const int64_t nn = c->nn;
  // node -> (element, local node) adjacency, elements ascending
  std::vector<int64_t> nadj_ptr(nn + 1, 0);
  for (const Block& B : c->blocks)
    for (int64_t i = 0; i < B.ne * B.nnpe; ++i) nadj_ptr[c->conn[B.conn_off + i] + 1]++;
  for (int64_t n = 0; n < nn; ++n) nadj_ptr[n + 1] += nadj_ptr[n];
  if (c->ne_total >= (int64_t(1) << 27))
    return fail(c, FEC_ERR_UNSUPPORTED, "more than 2^27 elements (%lld)", (long long)c->ne_total);
  std::vector<uint32_t> nadj(nadj_ptr[nn]);
  {
    std::vector<int64_t> fill(nadj_ptr.begin(), nadj_ptr.end() - 1);
    for (const Block& B : c->blocks)
      for (int64_t e = 0; e < B.ne; ++e)
        for (int a = 0; a < B.nnpe; ++a) {
          const int32_t n = c->conn[B.conn_off + e * B.nnpe + a];
          nadj[fill[n]++] = uint32_t(((B.elem_start + e) << 5) | a);
        }
  }
  auto elem_nodes = [&](int64_t ge, int* nnpe) -> const int32_t* {
    size_t b = 0;
    while (b + 1 < c->blocks.size() && ge >= c->blocks[b + 1].elem_start) ++b;
    const Block& B = c->blocks[b];
    *nnpe = B.nnpe;
    return c->conn.data() + B.conn_off + (ge - B.elem_start) * B.nnpe;
  };
  // sorted unique neighbour lists (two passes: count, then fill)
  std::vector<int64_t> nbr_ptr(nn + 1, 0);
  int64_t max_nbr = 0;
#pragma omp parallel reduction(max : max_nbr)
  {
    std::vector<int32_t> tmp;
#pragma omp for schedule(dynamic, 4096)
    for (int64_t n = 0; n < nn; ++n) {
      tmp.clear();
      for (int64_t p = nadj_ptr[n]; p < nadj_ptr[n + 1]; ++p) {
        int A;
        const int32_t* ce = elem_nodes(nadj[p] >> 5, &A);
        tmp.insert(tmp.end(), ce, ce + A);
      }
      std::sort(tmp.begin(), tmp.end());
      const int64_t u = std::unique(tmp.begin(), tmp.end()) - tmp.begin();
      nbr_ptr[n + 1] = u;
      max_nbr = std::max(max_nbr, u);
    }
  }
  for (int64_t n = 0; n < nn; ++n) nbr_ptr[n + 1] += nbr_ptr[n];
  std::vector<int32_t> nbr(nbr_ptr[nn]);
  std::vector<int32_t> col_len(nn, 0);
  std::vector<int32_t> rowoff(nbr_ptr[nn]);
  int64_t bad_len = 0;
#pragma omp parallel reduction(max : bad_len)
  {
    std::vector<int32_t> tmp;
#pragma omp for schedule(dynamic, 4096)
    for (int64_t n = 0; n < nn; ++n) {
      tmp.clear();
      for (int64_t p = nadj_ptr[n]; p < nadj_ptr[n + 1]; ++p) {
        int A;
        const int32_t* ce = elem_nodes(nadj[p] >> 5, &A);
        tmp.insert(tmp.end(), ce, ce + A);
      }
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      int32_t L = 0;
      for (size_t r = 0; r < tmp.size(); ++r) {
        nbr[nbr_ptr[n] + r] = tmp[r];
        rowoff[nbr_ptr[n] + r] = L;
        L += __builtin_popcount(c->umask[tmp[r]]);
      }
      col_len[n] = L;
      bad_len = std::max<int64_t>(bad_len, L);
    }
  }
  if (bad_len >= 65535) return fail(c, FEC_ERR_UNSUPPORTED, "a node couples to %lld dofs (limit 65534)", (long long)bad_len);
  std::vector<uint8_t> fullnbr(nn, 0);
  // fast-path flag: the node and all the nodes it couples to are fully unknown
  {
    const uint8_t full = uint8_t((1u << c->nf) - 1u);
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < nn; ++n) {
      bool all = (c->umask[n] & 0x7f) == full;
      for (int64_t p = nbr_ptr[n]; all && p < nbr_ptr[n + 1]; ++p) all = (c->umask[nbr[p]] & 0x7f) == full;
      fullnbr[n] = all ? 1 : 0;
    }
  }
  std::vector<int64_t> col_base(nn, 0);
  int64_t nnz = 0;
  int max_cols = 0;
  for (int64_t n = 0; n < nn; ++n) {
    col_base[n] = nnz;
    const int nc = __builtin_popcount(c->umask[n]);
    nnz += int64_t(nc) * col_len[n];
    if (nc) max_cols = std::max(max_cols, nc * col_len[n]);
  }
  // element map: row offset of node conn[b] within node conn[a]'s columns
  int64_t epos_total = 0;
  for (const Block& B : c->blocks) epos_total += (B.ne * B.nnpe * B.nnpe + 3) & ~int64_t(3);
  std::vector<uint16_t> epos(epos_total);
  for (const Block& B : c->blocks) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      const int32_t* ce = c->conn.data() + B.conn_off + e * B.nnpe;
      for (int a = 0; a < B.nnpe; ++a) {
        const int32_t n = ce[a];
        const int32_t* lo = nbr.data() + nbr_ptr[n];
        const int32_t* hi = nbr.data() + nbr_ptr[n + 1];
        for (int b = 0; b < B.nnpe; ++b) {
          const int64_t r = std::lower_bound(lo, hi, ce[b]) - lo;
          epos[B.epos_off + (e * B.nnpe + a) * B.nnpe + b] = uint16_t(rowoff[nbr_ptr[n] + r]);
        }
      }
    }
  }
  const int acc_stride = std::max(2, (max_cols + 1) & ~1);
  if (size_t(acc_stride) * sizeof(double) > 200 * 1024)
    return fail(c, FEC_ERR_UNSUPPORTED, "a node's columns hold %d entries; the gather supports %d", max_cols,
                int(200 * 1024 / sizeof(double)));
  int rc;
  if ((rc = upload(c, c->d_nadj_ptr, nadj_ptr.data(), sizeof(int64_t) * nadj_ptr.size()))) return rc;
  if ((rc = upload(c, c->d_nadj, nadj.data(), sizeof(uint32_t) * nadj.size()))) return rc;
  if ((rc = upload(c, c->d_epos, epos.data(), sizeof(uint16_t) * epos.size()))) return rc;
  if ((rc = upload(c, c->d_col_base, col_base.data(), sizeof(int64_t) * col_base.size()))) return rc;
  if ((rc = upload(c, c->d_col_len, col_len.data(), sizeof(int32_t) * col_len.size()))) return rc;
  {
    std::vector<uint8_t> um2(c->umask);
    for (int64_t n = 0; n < nn; ++n)
      if (fullnbr[n]) um2[n] |= uint8_t(fec::UMASK_FULL_NBR);
    if ((rc = upload(c, c->d_umask, um2.data(), um2.size()))) return rc;
  }
  c->nbr_ptr = std::move(nbr_ptr);
  c->nbr = std::move(nbr);
  c->col_base = std::move(col_base);
  c->col_len = std::move(col_len);
  c->nnz = nnz;
  c->acc_stride = acc_stride;
  c->pattern_ready = true;
  if (nnz_out) *nnz_out = nnz;
  return ok(c);
}

int fec_set_single_launch(fec_ctx* c, int on) {
  if (!c) return FEC_ERR_ARG;
  c->single_launch = on != 0;
  return ok(c);
}

int fec_pattern_build_device(fec_ctx* c, int64_t* nnz_out, void* stream) {
  if (!c) return FEC_ERR_ARG;
  if (c->n_unknowns < 0) return fail(c, FEC_ERR_STATE, "fec_pattern_build_device before fec_dofs_set");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  if (c->blocks.size() > size_t(fec::PATTERN_MAX_BLOCKS))
    return fail(c, FEC_ERR_UNSUPPORTED, "the device symbolic phase takes at most %d element blocks",
                fec::PATTERN_MAX_BLOCKS);
  if (c->ne_total >= (int64_t(1) << 27))
    return fail(c, FEC_ERR_UNSUPPORTED, "more than 2^27 elements (%lld)", (long long)c->ne_total);
  cudaSetDevice(c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  invalidate_pattern(c);
  const int64_t nn = c->nn;
  const int64_t nent = int64_t(c->conn.size());
  fec::PatternBlocks PB{};
  PB.nblocks = int(c->blocks.size());
  int64_t epos_total = 0;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    PB.nnpe[b] = B.nnpe;
    PB.ne[b] = B.ne;
    PB.elem_start[b] = B.elem_start;
    PB.conn_off[b] = B.conn_off;
    PB.epos_off[b] = B.epos_off;
    epos_total += (B.ne * B.nnpe * B.nnpe + 3) & ~int64_t(3);
  }
  // scratch: counts/cursors (int32 nn), scan partials, flags
  DevBuf t_cnt, t_cur, t_scan, t_flags, t_w, t_rowoff, t_um;
  struct Frees {
    DevBuf* b[7];
    ~Frees() {
      for (DevBuf* x : b) x->release();
    }
  } frees{{&t_cnt, &t_cur, &t_scan, &t_flags, &t_w, &t_rowoff, &t_um}};
  const size_t scan_n = fec::pattern_scan_scratch(nn + 1);
  FEC_CUDA(c, cudaMalloc(&t_cnt.p, sizeof(int32_t) * size_t(nn + 1)));
  FEC_CUDA(c, cudaMalloc(&t_cur.p, sizeof(int32_t) * size_t(nn + 1)));
  FEC_CUDA(c, cudaMalloc(&t_scan.p, sizeof(int64_t) * scan_n));
  FEC_CUDA(c, cudaMalloc(&t_flags.p, sizeof(int) * 4));
  FEC_CUDA(c, cudaMalloc(&t_w.p, sizeof(int64_t) * size_t(nn + 1)));
  FEC_CUDA(c, cudaMalloc(&t_um.p, size_t(nn + 1)));
  int32_t* cnt = static_cast<int32_t*>(t_cnt.p);
  int32_t* cur = static_cast<int32_t*>(t_cur.p);
  int64_t* scan = static_cast<int64_t*>(t_scan.p);
  int* flags = static_cast<int*>(t_flags.p);  // [0] overflow, [1] max column length, [2] max entries of a node
  const uint8_t* um = static_cast<const uint8_t*>(c->d_umask.p);
  const int32_t* conn = static_cast<const int32_t*>(c->d_conn.p);
  FEC_CUDA(c, cudaMemsetAsync(flags, 0, sizeof(int) * 4, s));
  // node -> (element, local node) adjacency, elements ascending
  FEC_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * size_t(nn + 1), s));
  FEC_CUDA(c, fec::pattern_count_adjacency(conn, nent, cnt, s));
  int rc;
  if ((rc = ensure(c, c->d_nadj_ptr, sizeof(int64_t) * size_t(nn + 1)))) return rc;
  if ((rc = ensure(c, c->d_nadj, sizeof(uint32_t) * size_t(nent > 0 ? nent : 1)))) return rc;
  int64_t* adj_ptr = static_cast<int64_t*>(c->d_nadj_ptr.p);
  uint32_t* nadj = static_cast<uint32_t*>(c->d_nadj.p);
  FEC_CUDA(c, fec::pattern_scan(cnt, nullptr, nn, adj_ptr, scan, s));
  FEC_CUDA(c, cudaMemsetAsync(cur, 0, sizeof(int32_t) * size_t(nn + 1), s));
  FEC_CUDA(c, fec::pattern_fill_adjacency(PB, conn, adj_ptr, nn, cur, nadj, s));
  // neighbour counts and column lengths, then the lists
  if ((rc = ensure(c, c->d_col_len, sizeof(int32_t) * size_t(nn + 1)))) return rc;
  int32_t* col_len = static_cast<int32_t*>(c->d_col_len.p);
  FEC_CUDA(c, fec::pattern_neighbours(PB, conn, adj_ptr, nadj, nn, um, cnt, col_len, nullptr, nullptr, nullptr,
                                      flags, s));
  if ((rc = ensure(c, c->d_nbr_ptr, sizeof(int64_t) * size_t(nn + 1)))) return rc;
  int64_t* nbr_ptr = static_cast<int64_t*>(c->d_nbr_ptr.p);
  FEC_CUDA(c, fec::pattern_scan(cnt, nullptr, nn, nbr_ptr, scan, s));
  int64_t n_nbr = 0;
  int overflow = 0;
  FEC_CUDA(c, cudaMemcpyAsync(&n_nbr, nbr_ptr + nn, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEC_CUDA(c, cudaMemcpyAsync(&overflow, flags, sizeof(int), cudaMemcpyDeviceToHost, s));
  FEC_CUDA(c, cudaStreamSynchronize(s));
  if (overflow)
    return fail(c, FEC_ERR_UNSUPPORTED, "a node gathers more than %d element nodes; use fec_pattern_build",
                fec::PATTERN_CAND_CAP);
  if ((rc = ensure(c, c->d_nbr, sizeof(int32_t) * size_t(n_nbr > 0 ? n_nbr : 1)))) return rc;
  FEC_CUDA(c, cudaMalloc(&t_rowoff.p, sizeof(int32_t) * size_t(n_nbr > 0 ? n_nbr : 1)));
  int32_t* nbr = static_cast<int32_t*>(c->d_nbr.p);
  int32_t* rowoff = static_cast<int32_t*>(t_rowoff.p);
  FEC_CUDA(c, fec::pattern_neighbours(PB, conn, adj_ptr, nadj, nn, um, cnt, col_len, nbr_ptr, nbr, rowoff, flags, s));
  // column sizes and offsets
  int64_t* w = static_cast<int64_t*>(t_w.p);
  FEC_CUDA(c, fec::pattern_column_sizes(nn, um, col_len, w, flags + 1, flags + 2, s));
  if ((rc = ensure(c, c->d_col_base, sizeof(int64_t) * size_t(nn + 1)))) return rc;
  int64_t* col_base = static_cast<int64_t*>(c->d_col_base.p);
  FEC_CUDA(c, fec::pattern_scan(nullptr, w, nn, col_base, scan, s));
  int host_flags[4] = {0, 0, 0, 0};
  int64_t nnz = 0;
  FEC_CUDA(c, cudaMemcpyAsync(host_flags, flags, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
  FEC_CUDA(c, cudaMemcpyAsync(&nnz, col_base + nn, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FEC_CUDA(c, cudaStreamSynchronize(s));
  if (host_flags[1] >= 65535)
    return fail(c, FEC_ERR_UNSUPPORTED, "a node couples to %d dofs (limit 65534)", host_flags[1]);
  const int max_cols = host_flags[2];
  const int acc_stride = std::max(2, (max_cols + 1) & ~1);
  if (size_t(acc_stride) * sizeof(double) > 200 * 1024)
    return fail(c, FEC_ERR_UNSUPPORTED, "a node's columns hold %d entries; the gather supports %d", max_cols,
                int(200 * 1024 / sizeof(double)));
  // element map and the full-neighbourhood flag
  if ((rc = ensure(c, c->d_epos, sizeof(uint16_t) * size_t(epos_total > 0 ? epos_total : 1)))) return rc;
  FEC_CUDA(c, fec::pattern_element_map(PB, conn, nbr_ptr, nbr, rowoff, static_cast<uint16_t*>(c->d_epos.p), s));
  uint8_t* um2 = static_cast<uint8_t*>(t_um.p);
  FEC_CUDA(c, fec::pattern_full_neighbourhood(nn, c->nf, nbr_ptr, nbr, um, uint8_t(fec::UMASK_FULL_NBR), um2, s));
  if (nn > 0) FEC_CUDA(c, cudaMemcpyAsync(c->d_umask.p, um2, size_t(nn), cudaMemcpyDeviceToDevice, s));
  // host copies for fec_pattern_get and the solver
  c->nbr_ptr.resize(size_t(nn + 1));
  c->nbr.resize(size_t(n_nbr));
  c->col_base.resize(size_t(nn));
  c->col_len.resize(size_t(nn));
  FEC_CUDA(c, cudaMemcpyAsync(c->nbr_ptr.data(), nbr_ptr, sizeof(int64_t) * size_t(nn + 1), cudaMemcpyDeviceToHost, s));
  if (n_nbr > 0)
    FEC_CUDA(c, cudaMemcpyAsync(c->nbr.data(), nbr, sizeof(int32_t) * size_t(n_nbr), cudaMemcpyDeviceToHost, s));
  if (nn > 0) {
    FEC_CUDA(c, cudaMemcpyAsync(c->col_base.data(), col_base, sizeof(int64_t) * size_t(nn), cudaMemcpyDeviceToHost, s));
    FEC_CUDA(c, cudaMemcpyAsync(c->col_len.data(), col_len, sizeof(int32_t) * size_t(nn), cudaMemcpyDeviceToHost, s));
  }
  FEC_CUDA(c, cudaStreamSynchronize(s));
  c->nnz = nnz;
  c->acc_stride = acc_stride;
  c->pattern_ready = true;
  if (nnz_out) *nnz_out = nnz;
  return ok(c);
}

int fec_pattern_get_device(const fec_ctx* cc, int64_t* colptr_dev, int64_t* rowval_dev, void* stream) {
  fec_ctx* c = const_cast<fec_ctx*>(cc);
  if (!c) return FEC_ERR_ARG;
  if (!c->pattern_ready) return fail(c, FEC_ERR_STATE, "fec_pattern_get_device before a pattern build");
  if (!colptr_dev || (!rowval_dev && c->nnz > 0)) return fail(c, FEC_ERR_ARG, "colptr or rowval is NULL");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  cudaSetDevice(c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc;
  if (!c->d_nbr_ptr.p) {  // a host-built pattern: its neighbour lists go up once
    if ((rc = upload(c, c->d_nbr_ptr, c->nbr_ptr.data(), sizeof(int64_t) * c->nbr_ptr.size()))) return rc;
    if ((rc = upload(c, c->d_nbr, c->nbr.data(), sizeof(int32_t) * c->nbr.size()))) return rc;
  }
  FEC_CUDA(c, fec::pattern_csc(c->nn, c->nf, static_cast<const uint8_t*>(c->d_umask.p),
                               static_cast<const int64_t*>(c->d_dtu.p), static_cast<const int64_t*>(c->d_nbr_ptr.p),
                               static_cast<const int32_t*>(c->d_nbr.p), static_cast<const int64_t*>(c->d_col_base.p),
                               static_cast<const int32_t*>(c->d_col_len.p), colptr_dev, rowval_dev, s));
  return ok(c);
}

int fec_pattern_get(const fec_ctx* cc, int64_t* colptr, int64_t* rowval) {
  fec_ctx* c = const_cast<fec_ctx*>(cc);
  if (!c) return FEC_ERR_ARG;
  if (!c->pattern_ready) return fail(c, FEC_ERR_STATE, "fec_pattern_get before fec_pattern_build");
  const int nf = c->nf;
  if (colptr) {
    colptr[0] = 1;
    for (int64_t n = 0; n < c->nn; ++n) {
      int kk = 0;
      for (int k = 0; k < nf; ++k) {
        if (!((c->umask[n] >> k) & 1)) continue;
        const int64_t col = c->dof_to_unknown[n * nf + k];
        colptr[col + 1] = c->col_base[n] + int64_t(kk + 1) * c->col_len[n] + 1;
        ++kk;
      }
    }
  }
  if (rowval) {
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t n = 0; n < c->nn; ++n) {
      const int nc = __builtin_popcount(c->umask[n]);
      int64_t w = c->col_base[n];
      for (int kk = 0; kk < nc; ++kk)
        for (int64_t p = c->nbr_ptr[n]; p < c->nbr_ptr[n + 1]; ++p) {
          const int32_t m = c->nbr[p];
          for (int i = 0; i < nf; ++i)
            if ((c->umask[m] >> i) & 1) rowval[w++] = c->dof_to_unknown[int64_t(m) * nf + i] + 1;
        }
    }
  }
  return ok(c);
}

int fec_update_field(fec_ctx* c, double* U, const double* Uu, int64_t num_bc, const int64_t* bc_dofs,
                     const double* bc_vals, void* stream) {
  if (!c) return FEC_ERR_ARG;
  if (c->n_unknowns < 0) return fail(c, FEC_ERR_STATE, "fec_update_field before fec_dofs_set");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  if (!U) return fail(c, FEC_ERR_ARG, "U is NULL");
  if (num_bc < 0 || (num_bc > 0 && (!bc_dofs || !bc_vals))) return fail(c, FEC_ERR_ARG, "bad Dirichlet arrays");
  cudaSetDevice(c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  c->n_timed = 0;
  LaunchTimer timer(c, s, "update_field");
  if (num_bc > 0) {
    set_dirichlet_kernel<<<unsigned((num_bc + 255) / 256), 256, 0, s>>>(U, num_bc, bc_dofs, bc_vals);
    FEC_CUDA(c, cudaGetLastError());
  }
  if (c->n_unknowns > 0) {
    if (!Uu) return fail(c, FEC_ERR_ARG, "Uu is NULL");
    set_unknowns_kernel<<<unsigned((c->n_unknowns + 255) / 256), 256, 0, s>>>(
        U, c->n_unknowns, static_cast<const int64_t*>(c->d_unknown_dofs.p), Uu);
    FEC_CUDA(c, cudaGetLastError());
  }
  return ok(c);
}

int fec_assemble(fec_ctx* c, int want, int precision, double t, double dt, const double* U, const double* U_old,
                 const double* state_old, double* state_new, double* R_u, double* nzval, void* stream) {
  (void)t;
  (void)dt;
  (void)U_old;
  if (!c) return FEC_ERR_ARG;
  c->last_launches = 0;
  if (!c->pattern_ready) return fail(c, FEC_ERR_STATE, "fec_assemble before fec_pattern_build");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  if (precision != FEC_FP64 && precision != FEC_FP32_ELEMENT)
    return fail(c, FEC_ERR_ARG, "unknown precision %d", precision);
  const bool want_r = (want & FEC_WANT_RESIDUAL) != 0, want_k = (want & FEC_WANT_STIFFNESS) != 0;
  if (!want_r && !want_k) return ok(c);
  if (!U) return fail(c, FEC_ERR_ARG, "U is NULL");
  if (want_r && !R_u && c->n_unknowns > 0) return fail(c, FEC_ERR_ARG, "R_u is NULL");
  if (want_k && !nzval && c->nnz > 0) return fail(c, FEC_ERR_ARG, "nzval is NULL");
  bool any_state = false;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    if (!B.physics) return fail(c, FEC_ERR_STATE, "block %d has no physics", int(b) + 1);
    if (num_fields_of(B.physics) != c->nf)
      return fail(c, FEC_ERR_ARG, "block %d physics has %d fields but the dofs have %d", int(b) + 1,
                  num_fields_of(B.physics), c->nf);
    if (num_states_of(B.physics)) any_state = true;
  }
  if (any_state && !state_old) return fail(c, FEC_ERR_ARG, "state_old is NULL for a physics with state");
  cudaSetDevice(c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* wait_err = nullptr;
  FEC_CUDA(c, fec::wait_error_flag(&wait_err));
  if (c->n_timed > 1) c->n_timed = 0;  // keep a preceding fec_update_field timing
  const size_t rsz = precision == FEC_FP64 ? sizeof(double) : sizeof(float);
  // element kernels: one launch per block, or one for all blocks (fec_set_single_launch)
  // (a single-block system is one launch already, on its own kernel)
  bool mixed = c->single_launch && precision == FEC_FP64 && c->blocks.size() >= 2 &&
               c->blocks.size() <= size_t(fec::MIXED_MAX_BLOCKS) && !fp64_native_env();
  std::vector<int> mixed_types;
  std::vector<ElemArgs> mixed_args;
  for (const Block& B : c->blocks) {
    mixed = mixed && B.physics == c->blocks[0].physics;
    mixed_types.push_back(B.elem_type);
  }
  mixed = mixed && fec::mixed_launch_supported(c->blocks[0].physics, int(c->blocks.size()), mixed_types.data());
  // the workspace as the kernels that run write it (the single launch writes every K_e whole)
  int64_t ke_total = 0, re_total = 0;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    ke_total += ke_entries(c, b, precision, want_k, mixed);
    re_total += c->blocks[b].ne * c->nf * c->blocks[b].nnpe;
  }
  int rc;
  if (want_k && (rc = ensure(c, c->d_Ke, rsz * size_t(ke_total)))) return rc;
  if (want_r && (rc = ensure(c, c->d_Re, rsz * size_t(re_total)))) return rc;
  GatherArgs ga;
  memset(&ga, 0, sizeof ga);
  int64_t ke_off = 0, re_off = 0, st_off = 0;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    const int ndof = c->nf * B.nnpe;
    ElemArgs ea;
    memset(&ea, 0, sizeof ea);
    ea.conn = static_cast<const int32_t*>(c->d_conn.p) + B.conn_off;
    ea.ne = B.ne;
    ea.coords = static_cast<const double*>(c->d_coords.p);
    ea.U = U;
    ea.ref = static_cast<const double*>(c->d_ref.p) + c->ref_off[b];
    ea.wait_err = wait_err;
    ea.wait_budget = g_wait_budget;
    for (int i = 0; i < 8; ++i) ea.props[i] = B.props[i];
    const int ns = num_states_of(B.physics);
    ea.state_old = ns ? state_old + st_off : nullptr;
    ea.state_new = (ns && state_new) ? state_new + st_off : nullptr;
    ea.Ke = want_k ? static_cast<char*>(c->d_Ke.p) + rsz * size_t(ke_off) : nullptr;
    ea.Re = want_r ? static_cast<char*>(c->d_Re.p) + rsz * size_t(re_off) : nullptr;
    ea.closure = c->d_cl_args.p;
    ea.affine = affine_table(c, b, precision, mixed);
    ea.ke_pairs = fp64_pairs(c, b, precision, want_k, mixed) ? 1 : 0;
    if (B.physics == FEC_PHYS_J2_MLP && !ea.closure)
      return fail(c, FEC_ERR_STATE, "block %d uses the learned closure but fec_closure_set was not called", int(b) + 1);
    cudaError_t e = cudaSuccess;
    if (mixed) {
      mixed_args.push_back(ea);
    } else {
      static const char* kNames[5][9] = {
          {"", "", "", "", "", "", "", "", ""},
          {"", "element_poisson", "element_poisson_quad4", "", "", "", "element_poisson_tet4",
           "element_poisson_tet10", "element_poisson_hex27"},
          {"", "element_neohookean", "", "", "", "", "element_neohookean_tet4", "element_neohookean_tet10",
           "element_neohookean_hex27"},
          {"", "element_j2", "", "", "", "", "element_j2_tet4", "element_j2_tet10", "element_j2_hex27"},
          {"", "element_j2_mlp", "", "", "", "", "", "", ""}};
      if (tc_closure(B, precision)) {
        // tensor-core closure: point table and state, then the FP32 hex8 element kernel on it
        const size_t tbytes = sizeof(float) * fec::POINT_TABLE_STRIDE * size_t(B.ne) * 8;
        if (int rc = ensure(c, c->d_cl_table, tbytes)) return rc;
        fec::TcClosure tcl;
        tcl.image = static_cast<const unsigned char*>(c->d_cl_img.p);
        tcl.counters = static_cast<unsigned long long*>(c->d_cl_cnt.p);
        tcl.table = static_cast<float*>(c->d_cl_table.p);
        tcl.tol = c->cl_tol;
        {
          LaunchTimer timer(c, s, "closure_j2_mlp_tc");
          e = fec::launch_j2mlp_points_tc(ea, tcl, s, &c->last_launches);
        }
        if (e == cudaSuccess) {
          LaunchTimer timer(c, s, "element_j2_mlp");
          e = fec::launch_point_table_hex8(want_r, want_k, ea, tcl.table, s, &c->last_launches);
        }
      } else {
        LaunchTimer timer(c, s, kNames[B.physics][B.elem_type]);
        if (B.physics == FEC_PHYS_POISSON)
          e = fec::launch_poisson(B.elem_type, precision, want_r, want_k, ea, s, &c->last_launches);
        else
          e = fec::launch_mech(B.physics, B.elem_type, precision, want_r, want_k, ea, s, &c->last_launches);
      }
    }
    if (e == cudaErrorNotSupported)
      return fail(c, FEC_ERR_UNSUPPORTED, "block %d: physics %d on element type %d is not built", int(b) + 1,
                  B.physics, B.elem_type);
    if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "element kernel launch: %s", cudaGetErrorString(e));
    BlockInfo& bi = ga.blk[b];
    bi.elem_start = B.elem_start;
    bi.ke_off = ke_off;
    bi.re_off = re_off;
    bi.conn_off = B.conn_off;
    bi.epos_off = B.epos_off;
    bi.nnpe = B.nnpe;
    bi.ndof = ndof;
    // the hex8 mechanics kernels write the node-rows layout (the FP64 tensor-core
    // kernel the symmetric half), the class tensor-core kernels the symmetric half
    const bool pairs = ea.ke_pairs ||
                       (want_k && fec::class_tc_runs(B.physics, B.elem_type, precision, want_r, want_k, ea.affine != nullptr));
    bi.layout = pairs ? fec::KE_PAIRS
                      : (B.elem_type == FEC_HEX8 && (B.physics == FEC_PHYS_NEOHOOKEAN || B.physics == FEC_PHYS_J2 ||
                                                     tc_closure(B, precision)))
                            ? fec::KE_NODE_ROWS
                            : fec::KE_ROW_MAJOR;
    ke_off += ke_entries(c, b, precision, want_k, mixed);
    re_off += B.ne * ndof;
    st_off += int64_t(ns) * B.nq * B.ne;
  }
  if (mixed) {
    if (int rc = ensure(c, c->d_tile_counter, sizeof(unsigned))) return rc;
    cudaError_t e;
    {
      LaunchTimer timer(c, s, "element_all_blocks");
      e = fec::launch_mech_mixed(c->blocks[0].physics, int(c->blocks.size()), mixed_types.data(), mixed_args.data(),
                                 want_r, want_k, static_cast<unsigned*>(c->d_tile_counter.p), s, &c->last_launches);
    }
    if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "element kernel launch: %s", cudaGetErrorString(e));
  }
  ga.nn = c->nn;
  ga.nf = c->nf;
  ga.nblocks = int(c->blocks.size());
  ga.nadj_ptr = static_cast<const int64_t*>(c->d_nadj_ptr.p);
  ga.nadj = static_cast<const uint32_t*>(c->d_nadj.p);
  ga.conn = static_cast<const int32_t*>(c->d_conn.p);
  ga.epos = static_cast<const uint16_t*>(c->d_epos.p);
  ga.umask = static_cast<const uint8_t*>(c->d_umask.p);
  ga.col_base = static_cast<const int64_t*>(c->d_col_base.p);
  ga.col_len = static_cast<const int32_t*>(c->d_col_len.p);
  ga.dof_to_unknown = static_cast<const int64_t*>(c->d_dtu.p);
  ga.Ke = c->d_Ke.p;
  ga.Re = c->d_Re.p;
  ga.nzval = want_k ? nzval : nullptr;
  ga.R_u = want_r ? R_u : nullptr;
  ga.acc_stride = c->acc_stride;
  cudaError_t e;
  // meshes of mixed element sizes: one gather launch per group of nodes of one size
  bool mixed_sizes = false;
  for (const Block& B : c->blocks) mixed_sizes = mixed_sizes || B.nnpe != c->blocks[0].nnpe;
  if (mixed_sizes && !gather_runs_generic() && !c->groups_ready)
    if (int rc = build_node_groups(c)) return rc;
  {
    LaunchTimer timer(c, s, "node_gather");
    if (mixed_sizes && !gather_runs_generic())
      e = fec::launch_gather_groups(precision, c->nf, ga, static_cast<const int32_t*>(c->d_node_groups.p),
                                    c->node_groups.data(), int(c->node_groups.size()), s, &c->last_launches);
    else
      e = fec::launch_gather(precision, c->nf, ga, s, &c->last_launches);
  }
  if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "gather launch: %s", cudaGetErrorString(e));
  return ok(c);
}

int fec_assemble_action(fec_ctx* c, int precision, double t, double dt, const double* U, const double* state_old,
                        const double* Vu, double* Kv_u, void* stream) {
  (void)t;
  (void)dt;
  if (!c) return FEC_ERR_ARG;
  c->last_launches = 0;
  if (!c->pattern_ready) return fail(c, FEC_ERR_STATE, "fec_assemble_action before fec_pattern_build");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  if (precision != FEC_FP64 && precision != FEC_FP32_ELEMENT)
    return fail(c, FEC_ERR_ARG, "unknown precision %d", precision);
  if (!U) return fail(c, FEC_ERR_ARG, "U is NULL");
  if (c->n_unknowns > 0 && (!Vu || !Kv_u)) return fail(c, FEC_ERR_ARG, "Vu or Kv_u is NULL");
  bool any_state = false;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    if (!B.physics) return fail(c, FEC_ERR_STATE, "block %d has no physics", int(b) + 1);
    if (num_fields_of(B.physics) != c->nf)
      return fail(c, FEC_ERR_ARG, "block %d physics has %d fields but the dofs have %d", int(b) + 1,
                  num_fields_of(B.physics), c->nf);
    if (num_states_of(B.physics)) any_state = true;
  }
  if (any_state && !state_old) return fail(c, FEC_ERR_ARG, "state_old is NULL for a physics with state");
  cudaSetDevice(c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* wait_err = nullptr;
  FEC_CUDA(c, fec::wait_error_flag(&wait_err));
  c->n_timed = 0;
  const size_t rsz = precision == FEC_FP64 ? sizeof(double) : sizeof(float);
  int64_t re_total = 0;
  for (const Block& B : c->blocks) re_total += B.ne * c->nf * B.nnpe;
  int rc;
  if ((rc = ensure(c, c->d_Re, rsz * size_t(re_total)))) return rc;
  // the direction as a full field: the unknowns' values, zero on Dirichlet dofs
  const int64_t ndofs = c->nn * c->nf;
  if ((rc = ensure(c, c->d_V, sizeof(double) * size_t(ndofs)))) return rc;
  double* V = static_cast<double*>(c->d_V.p);
  FEC_CUDA(c, cudaMemsetAsync(V, 0, sizeof(double) * size_t(ndofs), s));
  if (c->n_unknowns > 0) {
    set_unknowns_kernel<<<unsigned((c->n_unknowns + 255) / 256), 256, 0, s>>>(
        V, c->n_unknowns, static_cast<const int64_t*>(c->d_unknown_dofs.p), Vu);
    FEC_CUDA(c, cudaGetLastError());
    ++c->last_launches;
  }
  GatherArgs ga;
  memset(&ga, 0, sizeof ga);
  int64_t re_off = 0, st_off = 0;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    const int ndof = c->nf * B.nnpe;
    ElemArgs ea;
    memset(&ea, 0, sizeof ea);
    ea.conn = static_cast<const int32_t*>(c->d_conn.p) + B.conn_off;
    ea.ne = B.ne;
    ea.coords = static_cast<const double*>(c->d_coords.p);
    ea.U = U;
    ea.ref = static_cast<const double*>(c->d_ref.p) + c->ref_off[b];
    ea.wait_err = wait_err;
    ea.wait_budget = g_wait_budget;
    for (int i = 0; i < 8; ++i) ea.props[i] = B.props[i];
    const int ns = num_states_of(B.physics);
    ea.state_old = ns ? state_old + st_off : nullptr;
    ea.Re = static_cast<char*>(c->d_Re.p) + rsz * size_t(re_off);
    // FP64 blocks of translated hex8 elements: the block's constant gradients and JxW
    if (B.elem_type == FEC_HEX8 && precision == FEC_FP64 && B.congruent)
      if (const void* tab = affine_table(c, b, precision, false))
        ea.affine = static_cast<const unsigned char*>(tab) + fec::hex8_affine_grad_offset();
    cudaError_t e;
    {
      LaunchTimer timer(c, s, "element_action");
      e = fec::launch_action(B.physics, B.elem_type, precision, ea, V, s, &c->last_launches);
    }
    if (e == cudaErrorNotSupported)
      return fail(c, FEC_ERR_UNSUPPORTED, "block %d: matrix-free action of physics %d on element type %d is not built",
                  int(b) + 1, B.physics, B.elem_type);
    if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "action kernel launch: %s", cudaGetErrorString(e));
    BlockInfo& bi = ga.blk[b];
    bi.elem_start = B.elem_start;
    bi.ke_off = 0;
    bi.re_off = re_off;
    bi.conn_off = B.conn_off;
    bi.epos_off = B.epos_off;
    bi.nnpe = B.nnpe;
    bi.ndof = ndof;
    bi.layout = fec::KE_ROW_MAJOR;
    re_off += B.ne * ndof;
    st_off += int64_t(ns) * B.nq * B.ne;
  }
  ga.nn = c->nn;
  ga.nf = c->nf;
  ga.nblocks = int(c->blocks.size());
  ga.nadj_ptr = static_cast<const int64_t*>(c->d_nadj_ptr.p);
  ga.nadj = static_cast<const uint32_t*>(c->d_nadj.p);
  ga.conn = static_cast<const int32_t*>(c->d_conn.p);
  ga.epos = static_cast<const uint16_t*>(c->d_epos.p);
  ga.umask = static_cast<const uint8_t*>(c->d_umask.p);
  ga.col_base = static_cast<const int64_t*>(c->d_col_base.p);
  ga.col_len = static_cast<const int32_t*>(c->d_col_len.p);
  ga.dof_to_unknown = static_cast<const int64_t*>(c->d_dtu.p);
  ga.Re = c->d_Re.p;
  ga.nzval = nullptr;
  ga.R_u = Kv_u;
  ga.acc_stride = c->acc_stride;
  cudaError_t e;
  {
    LaunchTimer timer(c, s, "node_gather");
    e = fec::launch_gather(precision, c->nf, ga, s, &c->last_launches);
  }
  if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "gather launch: %s", cudaGetErrorString(e));
  return ok(c);
}

int fec_cg_solve(fec_ctx* c, const double* nzval, const double* b, double* x, int max_iter, double rtol,
                 int preconditioner, int* iterations, double* rel_residual, void* stream) {
  if (!c) return FEC_ERR_ARG;
  if (!c->pattern_ready) return fail(c, FEC_ERR_STATE, "fec_cg_solve before fec_pattern_build");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  if (c->n_unknowns > 0 && (!nzval || !b || !x)) return fail(c, FEC_ERR_ARG, "nzval, b or x is NULL");
  if (max_iter < 0 || !(rtol >= 0.0) || (preconditioner != 0 && preconditioner != 1))
    return fail(c, FEC_ERR_ARG, "max_iter >= 0, rtol >= 0, preconditioner 0 (none) or 1 (Jacobi)");
  if (c->n_unknowns > INT32_MAX) return fail(c, FEC_ERR_UNSUPPORTED, "more than 2^31 unknowns");
  cudaSetDevice(c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t n = c->n_unknowns;
  int rc;
  if (!c->d_rowval32.p && c->nnz > 0) {  // the pattern, 0-based, once per pattern
    std::vector<int64_t> colptr(size_t(n) + 1);
    std::vector<int64_t> rv(size_t(c->nnz));
    if ((rc = fec_pattern_get(c, colptr.data(), rv.data()))) return rc;
    std::vector<int32_t> rv32(rv.size());
    for (size_t i = 0; i < rv.size(); ++i) rv32[i] = int32_t(rv[i] - 1);
    for (auto& v : colptr) v -= 1;
    if ((rc = upload(c, c->d_colptr0, colptr.data(), sizeof(int64_t) * colptr.size()))) return rc;
    if ((rc = upload(c, c->d_rowval32, rv32.data(), sizeof(int32_t) * rv32.size()))) return rc;
  }
  if ((rc = ensure(c, c->d_cg, sizeof(double) * fec::pcg_scratch_doubles(n)))) return rc;
  fec::CscSym A;
  A.n = n;
  A.colptr = static_cast<const int64_t*>(c->d_colptr0.p);
  A.rowval = static_cast<const int32_t*>(c->d_rowval32.p);
  A.val = nzval;
  int it = 0;
  double rr = 0.0;
  const cudaError_t e = fec::pcg(A, b, x, static_cast<double*>(c->d_cg.p), max_iter, rtol, 10, preconditioner == 1,
                                 &it, &rr, s);
  if (iterations) *iterations = it;
  if (rel_residual) *rel_residual = rr;
  if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "conjugate gradients: %s", cudaGetErrorString(e));
  return ok(c);
}

int fec_check_finite(fec_ctx* c, const double* R_u, const double* nzval, int64_t* first_bad, void* stream) {
  if (!c) return FEC_ERR_ARG;
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  if (!c->pattern_ready) return fail(c, FEC_ERR_STATE, "fec_check_finite before fec_pattern_build");
  cudaSetDevice(c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc;
  if ((rc = ensure(c, c->d_flag, 2 * sizeof(unsigned long long)))) return rc;
  unsigned long long* d = static_cast<unsigned long long*>(c->d_flag.p);
  FEC_CUDA(c, cudaMemsetAsync(d, 0xFF, 2 * sizeof(unsigned long long), s));
  if (R_u && c->n_unknowns > 0) first_nonfinite_kernel<<<1216, 256, 0, s>>>(R_u, c->n_unknowns, d);
  if (nzval && c->nnz > 0) first_nonfinite_kernel<<<1216, 256, 0, s>>>(nzval, c->nnz, d + 1);
  FEC_CUDA(c, cudaGetLastError());
  unsigned long long h[2];
  FEC_CUDA(c, cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, s));
  FEC_CUDA(c, cudaStreamSynchronize(s));
  const unsigned long long none = ~0ull;
  if (first_bad) *first_bad = h[0] != none ? int64_t(h[0]) : (h[1] != none ? int64_t(h[1]) : -1);
  // a bounded wait in an element kernel that gave up leaves outputs that may be wrong however finite
  // they are: reported first, as the cause
  int* wait_err = nullptr;
  FEC_CUDA(c, fec::wait_error_flag(&wait_err));
  int werr = 0;
  FEC_CUDA(c, cudaMemcpy(&werr, wait_err, sizeof werr, cudaMemcpyDeviceToHost));
  if (werr)
    return fail(c, FEC_ERR_DEVICE,
                "an element kernel gave up a bounded wait (tensor-core MMA or bulk table copy); the outputs are "
                "invalid until fec_tensor_core_status(1) clears the flag");
  if (h[0] != none) return fail(c, FEC_ERR_NONFINITE, "residual entry %lld is not finite", (long long)h[0]);
  if (h[1] != none) return fail(c, FEC_ERR_NONFINITE, "nzval entry %lld is not finite", (long long)h[1]);
  return ok(c);
}

int fec_closure_set(fec_ctx* c, const float* params, const float* norm, float tol) {
  if (!c) return FEC_ERR_ARG;
  if (!params || !norm || !(tol > 0.f)) return fail(c, FEC_ERR_ARG, "closure parameters, normalisation and tol > 0");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot hold a closure");
  cudaSetDevice(c->device);
  std::vector<__nv_bfloat16> w(fec::MLP_PARAMS);
  for (int i = 0; i < fec::MLP_PARAMS; ++i) w[i] = __float2bfloat16_rn(params[i]);
  int rc;
  if ((rc = upload(c, c->d_cl_w, w.data(), sizeof(__nv_bfloat16) * w.size()))) return rc;
  const int nn = 2 * fec::MLP_IN + 2 * fec::MLP_OUT;
  if ((rc = upload(c, c->d_cl_norm, norm, sizeof(float) * nn))) return rc;
  const unsigned long long zero[4] = {0, 0, 0, 0};
  if ((rc = upload(c, c->d_cl_cnt, zero, sizeof zero))) return rc;
  const std::vector<unsigned char> img = fec::pack_mlp_image(params, norm);
  if ((rc = upload(c, c->d_cl_img, img.data(), img.size()))) return rc;
  c->cl_tol = tol;
  fec::ClosureArgs a;
  a.W = static_cast<const __nv_bfloat16*>(c->d_cl_w.p);
  const float* nd = static_cast<const float*>(c->d_cl_norm.p);
  a.in_mean = nd;
  a.in_std = nd + fec::MLP_IN;
  a.out_mean = nd + 2 * fec::MLP_IN;
  a.out_std = nd + 2 * fec::MLP_IN + fec::MLP_OUT;
  a.counters = static_cast<unsigned long long*>(c->d_cl_cnt.p);
  a.tol = tol;
  if ((rc = upload(c, c->d_cl_args, &a, sizeof a))) return rc;
  return ok(c);
}

int fec_closure_stats(fec_ctx* c, int64_t* plastic, int64_t* fallbacks, int reset) {
  if (!c) return FEC_ERR_ARG;
  if (!c->d_cl_cnt.p) return fail(c, FEC_ERR_STATE, "no closure installed");
  cudaSetDevice(c->device);
  unsigned long long h[3];
  FEC_CUDA(c, cudaMemcpy(h, c->d_cl_cnt.p, sizeof h, cudaMemcpyDeviceToHost));
  if (plastic) *plastic = int64_t(h[0]);
  if (fallbacks) *fallbacks = int64_t(h[1]);
  if (h[2]) return fail(c, FEC_ERR_DEVICE, "closure kernel: a wait on the tensor cores gave up (results invalid)");
  if (reset) FEC_CUDA(c, cudaMemset(c->d_cl_cnt.p, 0, 2 * sizeof(unsigned long long)));
  return ok(c);
}

int fec_set_wait_budget(long long clocks) {
  if (clocks < 0) return FEC_ERR_ARG;
  g_wait_budget = clocks;
  return FEC_OK;
}

int fec_set_profiling(fec_ctx* c, int on) {
  if (!c) return FEC_ERR_ARG;
  c->profiling = on != 0;
  c->n_timed = 0;
  return ok(c);
}

int fec_kernel_times(fec_ctx* c, float* ms, int cap, char* names, size_t len) {
  if (!c) return FEC_ERR_ARG;
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context");
  std::string all;
  const int n = c->n_timed;
  for (int i = 0; i < n; ++i) {
    cudaError_t e = cudaEventSynchronize(c->events[2 * i + 1]);
    if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "cudaEventSynchronize: %s", cudaGetErrorString(e));
    float t = 0.f;
    e = cudaEventElapsedTime(&t, c->events[2 * i], c->events[2 * i + 1]);
    if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "cudaEventElapsedTime: %s", cudaGetErrorString(e));
    if (ms && i < cap) ms[i] = t;
    if (i) all += ",";
    all += c->ev_names[i];
  }
  if (names && len) {
    strncpy(names, all.c_str(), len - 1);
    names[len - 1] = 0;
  }
  ok(c);
  return n;
}

}  // extern "C"

namespace {
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = T(tid) * T(1e-9) + T(k);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[tid] = s;
}
template <typename T>
int probe(int device, int iters, double* tflops) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return FEC_ERR_CUDA;
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return FEC_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_probe_kernel<T><<<blocks, threads>>>(out, 16, T(0.999), T(1e-3));
  cudaEventRecord(e0);
  fma_probe_kernel<T><<<blocks, threads>>>(out, iters, T(0.999), T(1e-3));
  cudaEventRecord(e1);
  cudaError_t st = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (st != cudaSuccess || ms <= 0.f) return FEC_ERR_CUDA;
  *tflops = 2.0 * double(blocks) * threads * iters * 8 / (double(ms) * 1e-3) / 1e12;
  return FEC_OK;
}

// df64_split and widen over an array: the device-side conversions of the FP64
// path, exposed so that tests can check them against host arithmetic.
__global__ void df64_split_check_kernel(const double* x, int64_t n, float* split, double* widened) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 s = fec::df64_split(x[i]);
  split[2 * i] = s.x;
  split[2 * i + 1] = s.y;
  widened[2 * i] = fec::widen(s.x);
  widened[2 * i + 1] = fec::widen(s.y);
}
}  // namespace

extern "C" {

int fec_df64_split_check(const double* x_dev, int64_t n, float* split_dev, double* widened_dev, void* stream) {
  if (n < 0 || (n > 0 && (!x_dev || !split_dev || !widened_dev))) return FEC_ERR_ARG;
  if (n == 0) return FEC_OK;
  const int threads = 256;
  const unsigned blocks = unsigned((n + threads - 1) / threads);
  df64_split_check_kernel<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(x_dev, n, split_dev, widened_dev);
  return cudaGetLastError() == cudaSuccess ? FEC_OK : FEC_ERR_CUDA;
}

int fec_probe_fma_rate(int device, int precision, double* tflops) {
  if (!tflops) return FEC_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return FEC_ERR_CUDA;
  if (precision == FEC_FP64) return probe<double>(device, 4000, tflops);
  if (precision == FEC_FP32_ELEMENT) return probe<float>(device, 40000, tflops);
  return FEC_ERR_ARG;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Assembly without device allocation.
//
// fec_assemble keeps its element-matrix workspace in context memory that it
// cudaMallocs on first use (and grows).  Some callers cannot let a library do
// that: applications that route every device allocation through their own pool
// (CUDA.jl's memory pool, PyTorch's caching allocator) and must not see memory
// appear outside the pool's accounting or a cudaFree synchronize the device in
// the middle of their step, and callers that fix their device-memory budget up
// front.  fec_assemble_noalloc does the same work with its workspace in the
// statically sized device array below, which the CUDA module reserves when the
// library is loaded on a device and keeps until the process exits.
// ---------------------------------------------------------------------------
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[FEC_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device `dev` (host code
// cannot use the symbol itself as a pointer).  Looked up again on every call
// made outside stream capture: a reset of the device's primary context
// (cudaDeviceReset, CUDA.jl's device_reset!) unloads the module, and the array
// can sit at another address once it is loaded again.  Under capture, where
// the lookup (which may load the module) is not allowed, the address of the
// last call on this device is used.
int noalloc_scratch_address(fec_ctx* c, int dev, cudaStream_t s, void** out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(c, FEC_ERR_ARG, "device %d out of range for the static scratch", dev);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();  // the failed query is not sticky; reset the runtime's last error
    cs = cudaStreamCaptureStatusActive;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(c, FEC_ERR_CUDA, "cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
    g_noalloc_addr[dev] = p;
  } else if (!g_noalloc_addr[dev]) {
    return fail(c, FEC_ERR_STATE,
                "fec_assemble_noalloc: the first call on a device must come before any stream capture");
  }
  *out = g_noalloc_addr[dev];
  return FEC_OK;
}

}  // namespace

extern "C" {

int fec_assemble_noalloc(fec_ctx* c, int want, int precision, double t, double dt, const double* U,
                         const double* U_old, const double* state_old, double* state_new, double* R_u, double* nzval,
                         void* stream) {
  (void)t;
  (void)dt;
  (void)U_old;
  if (!c) return FEC_ERR_ARG;
  c->last_launches = 0;
  if (!c->pattern_ready) return fail(c, FEC_ERR_STATE, "fec_assemble_noalloc before fec_pattern_build");
  if (c->device < 0) return fail(c, FEC_ERR_STATE, "host-only context (device -1) cannot run kernels");
  if (precision != FEC_FP64 && precision != FEC_FP32_ELEMENT)
    return fail(c, FEC_ERR_ARG, "unknown precision %d", precision);
  const bool want_r = (want & FEC_WANT_RESIDUAL) != 0, want_k = (want & FEC_WANT_STIFFNESS) != 0;
  if (!want_r && !want_k) return ok(c);
  if (!U) return fail(c, FEC_ERR_ARG, "U is NULL");
  if (want_r && !R_u && c->n_unknowns > 0) return fail(c, FEC_ERR_ARG, "R_u is NULL");
  if (want_k && !nzval && c->nnz > 0) return fail(c, FEC_ERR_ARG, "nzval is NULL");
  bool any_state = false;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    if (!B.physics) return fail(c, FEC_ERR_STATE, "block %d has no physics", int(b) + 1);
    if (num_fields_of(B.physics) != c->nf)
      return fail(c, FEC_ERR_ARG, "block %d physics has %d fields but the dofs have %d", int(b) + 1,
                  num_fields_of(B.physics), c->nf);
    if (num_states_of(B.physics)) any_state = true;
  }
  if (any_state && !state_old) return fail(c, FEC_ERR_ARG, "state_old is NULL for a physics with state");
  // workspace: element matrices, then (256-byte aligned) element residuals
  const size_t rsz = precision == FEC_FP64 ? sizeof(double) : sizeof(float);
  int64_t ke_total = 0, re_total = 0;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    ke_total += ke_entries(c, b, precision, want_k, false);
    re_total += c->blocks[b].ne * c->nf * c->blocks[b].nnpe;
  }
  const size_t ke_bytes = want_k ? rsz * size_t(ke_total) : 0;
  const size_t re_off_bytes = (ke_bytes + 255) & ~size_t(255);
  const size_t need = re_off_bytes + (want_r ? rsz * size_t(re_total) : 0);
  if (need > FEC_NOALLOC_SCRATCH_BYTES)
    return fail(c, FEC_ERR_ARG,
                "fec_assemble_noalloc needs %zu bytes of element workspace but the static scratch holds %zu "
                "(FEC_NOALLOC_SCRATCH_BYTES); use fec_assemble for this mesh",
                need, size_t(FEC_NOALLOC_SCRATCH_BYTES));
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, FEC_ERR_CUDA, "cudaSetDevice(%d) failed", c->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  int rc = noalloc_scratch_address(c, c->device, s, &scratch);
  if (rc) return rc;
  void* Ke = want_k ? scratch : nullptr;
  void* Re = want_r ? static_cast<char*>(scratch) + re_off_bytes : nullptr;
  int* wait_err = nullptr;
  FEC_CUDA(c, fec::wait_error_flag(&wait_err));
  c->n_timed = 0;  // no launch of this call is timed: the timing query reports none
  GatherArgs ga;
  memset(&ga, 0, sizeof ga);
  int64_t ke_off = 0, re_off = 0, st_off = 0;
  for (size_t b = 0; b < c->blocks.size(); ++b) {
    const Block& B = c->blocks[b];
    const int ndof = c->nf * B.nnpe;
    ElemArgs ea;
    memset(&ea, 0, sizeof ea);
    ea.conn = static_cast<const int32_t*>(c->d_conn.p) + B.conn_off;
    ea.ne = B.ne;
    ea.coords = static_cast<const double*>(c->d_coords.p);
    ea.U = U;
    ea.ref = static_cast<const double*>(c->d_ref.p) + c->ref_off[b];
    ea.wait_err = wait_err;
    ea.wait_budget = g_wait_budget;
    for (int i = 0; i < 8; ++i) ea.props[i] = B.props[i];
    const int ns = num_states_of(B.physics);
    ea.state_old = ns ? state_old + st_off : nullptr;
    ea.state_new = (ns && state_new) ? state_new + st_off : nullptr;
    ea.Ke = want_k ? static_cast<char*>(Ke) + rsz * size_t(ke_off) : nullptr;
    ea.Re = want_r ? static_cast<char*>(Re) + rsz * size_t(re_off) : nullptr;
    ea.closure = c->d_cl_args.p;
    ea.affine = affine_table(c, b, precision, false);
    ea.ke_pairs = fp64_pairs(c, b, precision, want_k, false) ? 1 : 0;
    if (B.physics == FEC_PHYS_J2_MLP && !ea.closure)
      return fail(c, FEC_ERR_STATE, "block %d uses the learned closure but fec_closure_set was not called", int(b) + 1);
    cudaError_t e;
    if (B.physics == FEC_PHYS_POISSON)
      e = fec::launch_poisson(B.elem_type, precision, want_r, want_k, ea, s, &c->last_launches);
    else
      e = fec::launch_mech(B.physics, B.elem_type, precision, want_r, want_k, ea, s, &c->last_launches);
    if (e == cudaErrorNotSupported)
      return fail(c, FEC_ERR_UNSUPPORTED, "block %d: physics %d on element type %d is not built", int(b) + 1,
                  B.physics, B.elem_type);
    if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "element kernel launch: %s", cudaGetErrorString(e));
    BlockInfo& bi = ga.blk[b];
    bi.elem_start = B.elem_start;
    bi.ke_off = ke_off;
    bi.re_off = re_off;
    bi.conn_off = B.conn_off;
    bi.epos_off = B.epos_off;
    bi.nnpe = B.nnpe;
    bi.ndof = ndof;
    // the hex8 mechanics kernels write the node-rows layout (the FP64 tensor-core
    // kernel the symmetric half), the class tensor-core kernels the symmetric half
    const bool pairs = ea.ke_pairs ||
                       (want_k && fec::class_tc_runs(B.physics, B.elem_type, precision, want_r, want_k, ea.affine != nullptr));
    bi.layout = pairs ? fec::KE_PAIRS
                      : (B.elem_type == FEC_HEX8 && (B.physics == FEC_PHYS_NEOHOOKEAN || B.physics == FEC_PHYS_J2))
                            ? fec::KE_NODE_ROWS
                            : fec::KE_ROW_MAJOR;
    ke_off += ke_entries(c, b, precision, want_k, false);
    re_off += B.ne * ndof;
    st_off += int64_t(ns) * B.nq * B.ne;
  }
  ga.nn = c->nn;
  ga.nf = c->nf;
  ga.nblocks = int(c->blocks.size());
  ga.nadj_ptr = static_cast<const int64_t*>(c->d_nadj_ptr.p);
  ga.nadj = static_cast<const uint32_t*>(c->d_nadj.p);
  ga.conn = static_cast<const int32_t*>(c->d_conn.p);
  ga.epos = static_cast<const uint16_t*>(c->d_epos.p);
  ga.umask = static_cast<const uint8_t*>(c->d_umask.p);
  ga.col_base = static_cast<const int64_t*>(c->d_col_base.p);
  ga.col_len = static_cast<const int32_t*>(c->d_col_len.p);
  ga.dof_to_unknown = static_cast<const int64_t*>(c->d_dtu.p);
  ga.Ke = Ke;
  ga.Re = Re;
  ga.nzval = want_k ? nzval : nullptr;
  ga.R_u = want_r ? R_u : nullptr;
  ga.acc_stride = c->acc_stride;
  cudaError_t e = fec::launch_gather(precision, c->nf, ga, s, &c->last_launches);
  if (e != cudaSuccess) return fail(c, FEC_ERR_CUDA, "gather launch: %s", cudaGetErrorString(e));
  return ok(c);
}

}  // extern "C"
