// fec_pattern.cu -- the symbolic phase on the device (see fec_pattern.h).
//
// Node adjacency is a counting sort (atomics for the counts and slots, then each
// node's short run sorted, so the order is the host's increasing element order
// whatever the atomics did).  Neighbour lists: one warp per node gathers the
// nodes of its adjacent elements into shared memory, sorts them (bitonic) and
// keeps the first of each run, with each kept neighbour's row offset (the
// unknown components before it) from a warp prefix sum.  Column lengths,
// offsets and the element map follow from these; sizes are int64 throughout.
#include <climits>
#include "fec_pattern.h"

namespace fec {
namespace {

constexpr int SCAN_BLOCK = 1024;
constexpr int NB_WARPS = 4;  // warps per block of the neighbour kernel

__device__ __forceinline__ int block_of(const PatternBlocks& B, int64_t ge) {
  int b = 0;
  while (b + 1 < B.nblocks && ge >= B.elem_start[b + 1]) ++b;
  return b;
}

__global__ void count_kernel(const int32_t* __restrict__ conn, int64_t n, int32_t* cnt) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[conn[i]], 1);
}

// ---- int64 exclusive scan: block sums, scan of the sums, block-local scans ------
__device__ __forceinline__ int64_t block_inclusive_scan(int64_t v, int64_t* s_warp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) s_warp[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < SCAN_BLOCK / 32 ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    s_warp[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  return v + (warp > 0 ? s_warp[warp - 1] : 0);
}

__device__ __forceinline__ int64_t scan_in(const int32_t* in32, const int64_t* in64, int64_t i, int64_t n) {
  if (i >= n) return 0;
  return in32 ? int64_t(in32[i]) : in64[i];
}

__global__ void __launch_bounds__(SCAN_BLOCK) scan_sums_kernel(const int32_t* in32, const int64_t* in64, int64_t n,
                                                               int64_t* sums) {
  __shared__ int64_t s_warp[32];
  const int64_t i = int64_t(blockIdx.x) * SCAN_BLOCK + threadIdx.x;
  const int64_t v = block_inclusive_scan(scan_in(in32, in64, i, n), s_warp);
  if (threadIdx.x == SCAN_BLOCK - 1) sums[blockIdx.x] = v;
}

__global__ void __launch_bounds__(SCAN_BLOCK) scan_offsets_kernel(int64_t* sums, int64_t nb) {
  __shared__ int64_t s_warp[32];
  __shared__ int64_t s_total;
  int64_t carry = 0;
  for (int64_t c0 = 0; c0 < nb; c0 += SCAN_BLOCK) {
    const int64_t i = c0 + threadIdx.x;
    const int64_t v = i < nb ? sums[i] : 0;
    const int64_t inc = block_inclusive_scan(v, s_warp);
    if (i < nb) sums[i] = carry + inc - v;  // exclusive
    if (threadIdx.x == SCAN_BLOCK - 1) s_total = inc;
    __syncthreads();
    carry += s_total;
    __syncthreads();  // s_total and s_warp are rewritten by the next chunk
  }
}

__global__ void __launch_bounds__(SCAN_BLOCK) scan_final_kernel(const int32_t* in32, const int64_t* in64, int64_t n,
                                                                const int64_t* offs, int64_t* out) {
  __shared__ int64_t s_warp[32];
  const int64_t i = int64_t(blockIdx.x) * SCAN_BLOCK + threadIdx.x;
  const int64_t inc = block_inclusive_scan(scan_in(in32, in64, i, n), s_warp);
  if (i < n) out[i + 1] = offs[blockIdx.x] + inc;
  if (i == 0) out[0] = 0;
}

// ---- adjacency -------------------------------------------------------------------
__global__ void fill_kernel(const int32_t* __restrict__ conn, int64_t ne, int nnpe, int64_t elem_start,
                            const int64_t* __restrict__ ptr, int32_t* cursor, uint32_t* nadj) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= ne * nnpe) return;
  const int64_t e = i / nnpe;
  const int a = int(i - e * nnpe);
  const int32_t n = conn[i];
  const int64_t pos = ptr[n] + atomicAdd(&cursor[n], 1);
  nadj[pos] = uint32_t(((elem_start + e) << 5) | a);
}

__global__ void sort_runs_kernel(const int64_t* __restrict__ ptr, int64_t nn, uint32_t* nadj) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int64_t lo = ptr[n], hi = ptr[n + 1];
  for (int64_t p = lo + 1; p < hi; ++p) {  // insertion sort: runs are a few to a few tens long
    const uint32_t v = nadj[p];
    int64_t q = p - 1;
    while (q >= lo && nadj[q] > v) {
      nadj[q + 1] = nadj[q];
      --q;
    }
    nadj[q + 1] = v;
  }
}

// ---- neighbour lists (warp per node) ------------------------------------------------
template <bool FILL>
__global__ void __launch_bounds__(NB_WARPS * 32)
    neighbours_kernel(PatternBlocks B, const int32_t* __restrict__ conn, const int64_t* __restrict__ adj_ptr,
                      const uint32_t* __restrict__ nadj, int64_t nn, const uint8_t* __restrict__ umask,
                      int32_t* nbr_cnt, int32_t* col_len, const int64_t* __restrict__ nbr_ptr, int32_t* nbr,
                      int32_t* rowoff, int* err) {
  __shared__ int32_t s_cand[NB_WARPS][PATTERN_CAND_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t n = int64_t(blockIdx.x) * NB_WARPS + warp;
  if (n >= nn) return;  // whole warps leave together
  int32_t* cand = s_cand[warp];
  const unsigned lt = (1u << lane) - 1u;
  const int64_t p0 = adj_ptr[n], p1 = adj_ptr[n + 1];
  int count = 0;
  bool overflow = false;
  for (int64_t c0 = p0; c0 < p1; c0 += 32) {
    const int64_t p = c0 + lane;
    int A = 0;
    const int32_t* ce = nullptr;
    if (p < p1) {
      const int64_t ge = int64_t(nadj[p] >> 5);
      const int b = block_of(B, ge);
      A = B.nnpe[b];
      ce = conn + B.conn_off[b] + (ge - B.elem_start[b]) * A;
    }
    int off = A;  // exclusive prefix of A over the lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, off, o);
      if (lane >= o) off += t;
    }
    const int total = __shfl_sync(0xffffffffu, off, 31);
    off -= A;
    if (count + total > PATTERN_CAND_CAP) {
      overflow = true;
      break;
    }
    for (int j = 0; j < A; ++j) cand[count + off + j] = ce[j];
    count += total;
  }
  if (overflow) {
    if (lane == 0) atomicExch(err, 1);
    return;
  }
  int P = 32;
  while (P < count) P <<= 1;
  for (int i = count + lane; i < P; i += 32) cand[i] = INT_MAX;
  __syncwarp();
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < P; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const int32_t x = cand[i], y = cand[ixj];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            cand[i] = y;
            cand[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
  int kept = 0, L = 0;
  for (int i0 = 0; i0 < count; i0 += 32) {
    const int i = i0 + lane;
    const int32_t v = i < count ? cand[i] : -1;
    const bool keep = i < count && (i == 0 || cand[i - 1] != v);
    const int w = keep ? __popc(umask[v] & 0x7fu) : 0;
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    int ws = w;  // inclusive prefix of w
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += t;
    }
    if (FILL && keep) {
      const int64_t slot = nbr_ptr[n] + kept + __popc(mask & lt);
      nbr[slot] = v;
      rowoff[slot] = L + ws - w;
    }
    kept += __popc(mask);
    L += __shfl_sync(0xffffffffu, ws, 31);
  }
  if (!FILL && lane == 0) {
    nbr_cnt[n] = kept;
    col_len[n] = L;
  }
}

__global__ void column_sizes_kernel(int64_t nn, const uint8_t* __restrict__ umask, const int32_t* __restrict__ col_len,
                                    int64_t* w, int* max_len, int* max_cols) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int nc = __popc(umask[n] & 0x7fu);
  const int64_t v = int64_t(nc) * col_len[n];
  w[n] = v;
  atomicMax(max_len, col_len[n]);
  if (nc) atomicMax(max_cols, int(v < INT_MAX ? v : INT_MAX));
}

__global__ void element_map_kernel(const int32_t* __restrict__ conn, int64_t ne, int nnpe,
                                   const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                                   const int32_t* __restrict__ rowoff, uint16_t* epos) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;  // (e, a)
  if (i >= ne * nnpe) return;
  const int64_t e = i / nnpe;
  const int32_t n = conn[i];
  const int64_t lo = nbr_ptr[n], hi = nbr_ptr[n + 1];
  for (int b = 0; b < nnpe; ++b) {
    const int32_t m = conn[e * nnpe + b];
    int64_t l = lo, h = hi;  // lower bound of m in nbr[lo, hi); m is there (it shares element e)
    while (l < h) {
      const int64_t mid = l + ((h - l) >> 1);
      if (nbr[mid] < m)
        l = mid + 1;
      else
        h = mid;
    }
    epos[i * nnpe + b] = uint16_t(l < hi ? rowoff[l] : 0);
  }
}

__global__ void full_neighbourhood_kernel(int64_t nn, int nf, const int64_t* __restrict__ nbr_ptr,
                                          const int32_t* __restrict__ nbr, const uint8_t* __restrict__ umask,
                                          uint8_t flag, uint8_t* out) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const unsigned full = (1u << nf) - 1u;
  const unsigned own = umask[n] & 0x7fu;
  bool all = own == full;
  for (int64_t p = nbr_ptr[n]; all && p < nbr_ptr[n + 1]; ++p) all = (umask[nbr[p]] & 0x7fu) == full;
  out[n] = uint8_t(own | (all ? flag : 0u));
}

__global__ void colptr_kernel(int64_t nn, int nf, const uint8_t* __restrict__ umask,
                              const int64_t* __restrict__ dtu, const int64_t* __restrict__ col_base,
                              const int32_t* __restrict__ col_len, int64_t* colptr) {
  const int64_t n = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (n == 0) colptr[0] = 1;
  if (n >= nn) return;
  const unsigned um = umask[n] & 0x7fu;
  int kk = 0;
  for (int k = 0; k < nf; ++k) {
    if (!((um >> k) & 1u)) continue;
    const int64_t col = dtu[n * nf + k];
    colptr[col + 1] = col_base[n] + int64_t(kk + 1) * col_len[n] + 1;
    ++kk;
  }
}

// One warp per node: lanes over the rows of the node's first column, the same
// rows repeated for its other columns.
__global__ void rowval_kernel(int64_t nn, int nf, const uint8_t* __restrict__ umask, const int64_t* __restrict__ dtu,
                              const int64_t* __restrict__ nbr_ptr, const int32_t* __restrict__ nbr,
                              const int64_t* __restrict__ col_base, const int32_t* __restrict__ col_len,
                              int64_t* rowval) {
  const int64_t n = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (n >= nn) return;
  const int nc = __popc(umask[n] & 0x7fu);
  if (nc == 0) return;
  const int64_t base = col_base[n], L = col_len[n];
  int64_t r = 0;  // rows written so far in the first column
  for (int64_t p0 = nbr_ptr[n]; p0 < nbr_ptr[n + 1]; p0 += 32) {
    const int64_t p = p0 + lane;
    const int32_t m = p < nbr_ptr[n + 1] ? nbr[p] : 0;
    const unsigned um = p < nbr_ptr[n + 1] ? (umask[m] & 0x7fu) : 0u;
    const int cnt = __popc(um);
    int pre = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, pre, o);
      if (lane >= o) pre += t;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 31);
    pre -= cnt;
    int j = 0;
    for (int i = 0; i < nf; ++i) {
      if (!((um >> i) & 1u)) continue;
      const int64_t v = dtu[int64_t(m) * nf + i] + 1;
      for (int kk = 0; kk < nc; ++kk) rowval[base + int64_t(kk) * L + r + pre + j] = v;
      ++j;
    }
    r += total;
  }
}

inline unsigned grid_of(int64_t n, int threads) { return unsigned((n + threads - 1) / threads); }

}  // namespace

cudaError_t pattern_count_adjacency(const int32_t* conn, int64_t n_entries, int32_t* cnt, cudaStream_t s) {
  if (n_entries > 0) count_kernel<<<grid_of(n_entries, 256), 256, 0, s>>>(conn, n_entries, cnt);
  return cudaGetLastError();
}

size_t pattern_scan_scratch(int64_t n) { return size_t((n + SCAN_BLOCK - 1) / SCAN_BLOCK + 1); }

cudaError_t pattern_scan(const int32_t* in32, const int64_t* in64, int64_t n, int64_t* out, int64_t* scratch,
                         cudaStream_t s) {
  if (n <= 0) return cudaMemsetAsync(out, 0, sizeof(int64_t), s);
  const int64_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
  scan_sums_kernel<<<unsigned(nb), SCAN_BLOCK, 0, s>>>(in32, in64, n, scratch);
  scan_offsets_kernel<<<1, SCAN_BLOCK, 0, s>>>(scratch, nb);
  scan_final_kernel<<<unsigned(nb), SCAN_BLOCK, 0, s>>>(in32, in64, n, scratch, out);
  return cudaGetLastError();
}

cudaError_t pattern_fill_adjacency(const PatternBlocks& B, const int32_t* conn, const int64_t* ptr, int64_t nn,
                                   int32_t* cursor, uint32_t* nadj, cudaStream_t s) {
  for (int b = 0; b < B.nblocks; ++b) {
    const int64_t n = B.ne[b] * B.nnpe[b];
    if (n > 0)
      fill_kernel<<<grid_of(n, 256), 256, 0, s>>>(conn + B.conn_off[b], B.ne[b], B.nnpe[b], B.elem_start[b], ptr,
                                                   cursor, nadj);
  }
  if (nn > 0) sort_runs_kernel<<<grid_of(nn, 256), 256, 0, s>>>(ptr, nn, nadj);
  return cudaGetLastError();
}

cudaError_t pattern_neighbours(const PatternBlocks& B, const int32_t* conn, const int64_t* adj_ptr,
                               const uint32_t* nadj, int64_t nn, const uint8_t* umask, int32_t* nbr_cnt,
                               int32_t* col_len, const int64_t* nbr_ptr, int32_t* nbr, int32_t* rowoff, int* err,
                               cudaStream_t s) {
  if (nn <= 0) return cudaSuccess;
  const unsigned grid = grid_of(nn, NB_WARPS);
  if (nbr)
    neighbours_kernel<true><<<grid, NB_WARPS * 32, 0, s>>>(B, conn, adj_ptr, nadj, nn, umask, nbr_cnt, col_len,
                                                           nbr_ptr, nbr, rowoff, err);
  else
    neighbours_kernel<false><<<grid, NB_WARPS * 32, 0, s>>>(B, conn, adj_ptr, nadj, nn, umask, nbr_cnt, col_len,
                                                            nbr_ptr, nbr, rowoff, err);
  return cudaGetLastError();
}

cudaError_t pattern_column_sizes(int64_t nn, const uint8_t* umask, const int32_t* col_len, int64_t* w, int* max_len,
                                 int* max_cols, cudaStream_t s) {
  if (nn > 0) column_sizes_kernel<<<grid_of(nn, 256), 256, 0, s>>>(nn, umask, col_len, w, max_len, max_cols);
  return cudaGetLastError();
}

cudaError_t pattern_element_map(const PatternBlocks& B, const int32_t* conn, const int64_t* nbr_ptr,
                                const int32_t* nbr, const int32_t* rowoff, uint16_t* epos, cudaStream_t s) {
  for (int b = 0; b < B.nblocks; ++b) {
    const int64_t n = B.ne[b] * B.nnpe[b];
    if (n > 0)
      element_map_kernel<<<grid_of(n, 256), 256, 0, s>>>(conn + B.conn_off[b], B.ne[b], B.nnpe[b], nbr_ptr, nbr,
                                                         rowoff, epos + B.epos_off[b]);
  }
  return cudaGetLastError();
}

cudaError_t pattern_full_neighbourhood(int64_t nn, int nf, const int64_t* nbr_ptr, const int32_t* nbr,
                                       const uint8_t* umask, uint8_t full_flag, uint8_t* umask_out, cudaStream_t s) {
  if (nn > 0)
    full_neighbourhood_kernel<<<grid_of(nn, 256), 256, 0, s>>>(nn, nf, nbr_ptr, nbr, umask, full_flag, umask_out);
  return cudaGetLastError();
}

cudaError_t pattern_csc(int64_t nn, int nf, const uint8_t* umask, const int64_t* dof_to_unknown,
                        const int64_t* nbr_ptr, const int32_t* nbr, const int64_t* col_base, const int32_t* col_len,
                        int64_t* colptr, int64_t* rowval, cudaStream_t s) {
  if (colptr) {
    const int64_t n = nn > 0 ? nn : 1;
    colptr_kernel<<<grid_of(n, 256), 256, 0, s>>>(nn, nf, umask, dof_to_unknown, col_base, col_len, colptr);
  }
  if (rowval && nn > 0)
    rowval_kernel<<<grid_of(nn * 32, 256), 256, 0, s>>>(nn, nf, umask, dof_to_unknown, nbr_ptr, nbr, col_base,
                                                        col_len, rowval);
  return cudaGetLastError();
}

}  // namespace fec
