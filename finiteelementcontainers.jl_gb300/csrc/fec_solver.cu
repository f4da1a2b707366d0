// fec_solver.cu -- the linear solve after assembly: preconditioned conjugate
// gradients on the assembled CSC stiffness over the unknowns (the reference's
// IterativeLinearSolver, src/Solvers.jl:88-152, which hands K and R to a Krylov
// CG), on the device.
//
// K is symmetric, so its CSC columns are its rows: y = K x takes one warp per
// column j, y_j = sum_p val[p] x[row[p]], reduced by a fixed shuffle tree.  Dot
// products reduce in two fixed-shape stages (per-block partials in a fixed grid,
// then one block), so a solve is bitwise repeatable.  The CG scalars live on the
// device; the host reads the residual norm every few iterations only.
#include <cmath>
#include <vector>
#include "fec_solver.h"

namespace fec {
namespace {

constexpr int DOT_BLOCKS = 608, DOT_THREADS = 256;

__global__ void spmv_sym_kernel(CscSym A, const double* __restrict__ x, double* __restrict__ y) {
  const int64_t j = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= A.n) return;
  double s = 0.0;
  for (int64_t p = A.colptr[j] + lane; p < A.colptr[j + 1]; p += 32) s = fma(A.val[p], x[A.rowval[p]], s);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) y[j] = s;
}

__global__ void inv_diag_kernel(CscSym A, double* __restrict__ inv_diag) {
  const int64_t j = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (j >= A.n) return;
  double d = 0.0;
  for (int64_t p = A.colptr[j] + lane; p < A.colptr[j + 1]; p += 32)
    if (A.rowval[p] == j) d = A.val[p];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
  if (lane == 0) inv_diag[j] = d != 0.0 ? 1.0 / d : 1.0;
}

__global__ void __launch_bounds__(DOT_THREADS) dot_partial_kernel(int64_t n, const double* __restrict__ a,
                                                                  const double* __restrict__ b,
                                                                  double* __restrict__ partial) {
  __shared__ double red[DOT_THREADS];
  const int64_t chunk = (n + DOT_BLOCKS - 1) / DOT_BLOCKS;
  const int64_t lo = int64_t(blockIdx.x) * chunk, hi = lo + chunk < n ? lo + chunk : n;
  double s = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += DOT_THREADS) s = fma(a[i], b[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = DOT_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(1024) dot_final_kernel(const double* __restrict__ partial, double* out) {
  __shared__ double red[1024];
  red[threadIdx.x] = threadIdx.x < DOT_BLOCKS ? partial[threadIdx.x] : 0.0;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// r = b - r (r holds K x on entry); z = M^-1 r; p = z
__global__ void cg_init_kernel(int64_t n, const double* b, double* r, double* z, double* p, const double* inv_diag) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ri = b[i] - r[i];
  r[i] = ri;
  const double zi = inv_diag ? inv_diag[i] * ri : ri;
  z[i] = zi;
  p[i] = zi;
}

// alpha = rz / pAp; x += alpha p; r -= alpha Ap; z = M^-1 r
__global__ void cg_update_kernel(int64_t n, const double* sc, double* x, double* r, double* z, const double* p,
                                 const double* Ap, const double* inv_diag) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double alpha = sc[0] / sc[1];
  x[i] = fma(alpha, p[i], x[i]);
  const double ri = fma(-alpha, Ap[i], r[i]);
  r[i] = ri;
  z[i] = inv_diag ? inv_diag[i] * ri : ri;
}

// beta = rz_new / rz; p = z + beta p
__global__ void cg_direction_kernel(int64_t n, const double* sc, const double* z, double* p) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = fma(sc[2] / sc[0], p[i], z[i]);
}

__global__ void copy_scalar_kernel(double* sc) { sc[0] = sc[2]; }

}  // namespace

size_t pcg_scratch_doubles(int64_t n) { return size_t(5) * size_t(n) + DOT_BLOCKS + 8; }

cudaError_t spmv_sym(const CscSym& A, const double* x, double* y, cudaStream_t s) {
  const int64_t threads = A.n * 32;
  spmv_sym_kernel<<<unsigned((threads + 255) / 256), 256, 0, s>>>(A, x, y);
  return cudaGetLastError();
}

cudaError_t pcg(const CscSym& A, const double* b, double* x, double* scratch, int max_iter, double rtol,
                int check_every, bool jacobi, int* iterations, double* rel_residual, cudaStream_t s) {
  const int64_t n = A.n;
  double* r = scratch;
  double* z = r + n;
  double* p = z + n;
  double* Ap = p + n;
  double* inv_diag = Ap + n;
  double* partial = inv_diag + n;
  double* sc = partial + DOT_BLOCKS;  // [0] rz, [1] pAp, [2] rz_new, [3] rr, [4] bb
  const unsigned gv = unsigned((n + 255) / 256);
  const unsigned gw = unsigned((n * 32 + 255) / 256);
  auto dot = [&](const double* a, const double* bb, double* out) {
    dot_partial_kernel<<<DOT_BLOCKS, DOT_THREADS, 0, s>>>(n, a, bb, partial);
    dot_final_kernel<<<1, 1024, 0, s>>>(partial, out);
  };
  *iterations = 0;
  *rel_residual = 0.0;
  if (n == 0) return cudaSuccess;
  if (jacobi) inv_diag_kernel<<<gw, 256, 0, s>>>(A, inv_diag);
  spmv_sym_kernel<<<gw, 256, 0, s>>>(A, x, r);
  cg_init_kernel<<<gv, 256, 0, s>>>(n, b, r, z, p, jacobi ? inv_diag : nullptr);
  dot(r, z, sc + 0);
  dot(b, b, sc + 4);
  double host[2] = {0.0, 0.0};
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(&host[1], sc + 4, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  const double bnorm = std::sqrt(host[1]);
  if (bnorm == 0.0) {
    cudaMemsetAsync(x, 0, sizeof(double) * size_t(n), s);
    return cudaGetLastError();
  }
  int it = 0;
  for (; it < max_iter;) {
    spmv_sym_kernel<<<gw, 256, 0, s>>>(A, p, Ap);
    dot(p, Ap, sc + 1);
    cg_update_kernel<<<gv, 256, 0, s>>>(n, sc, x, r, z, p, Ap, jacobi ? inv_diag : nullptr);
    ++it;
    if (it % check_every == 0 || it == max_iter) {
      dot(r, r, sc + 3);
      if ((e = cudaMemcpyAsync(&host[0], sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
      *rel_residual = std::sqrt(host[0]) / bnorm;
      if (*rel_residual <= rtol) break;
    }
    dot(r, z, sc + 2);
    cg_direction_kernel<<<gv, 256, 0, s>>>(n, sc, z, p);
    copy_scalar_kernel<<<1, 1, 0, s>>>(sc);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  *iterations = it;
  return cudaGetLastError();
}

}  // namespace fec
