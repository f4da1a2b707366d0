// fec_mixed.cu -- all element blocks of an FP64 mechanics system in one
// persistent launch.
//
// Blocks of different element types (hex8, tet4, tet10, hex27) have different
// kernels; here one kernel of 192-thread CTAs (three per SM) takes work tiles
// from one list over all blocks (dynamically: each CTA fetches its next tile
// from a device counter) and runs, per tile, the same tile function the per-block kernels use, in a tile shape of 192 threads: 8
// hex8 elements x 24 threads and one hex27 element x 192 threads (the shapes of
// their own kernels), 16 tet4 x 12, and 3 tet10 x 60 (two column chunks per
// row; the last 12 threads idle).  The arithmetic per element is the per-block
// kernels', so the workspace -- and the assembled system -- is bitwise the same.
// Blocks are ordered by the work of one tile, heaviest first, so that the light
// tiles fill the tail of the launch.
#include "fec_launch.h"
#include "fec_mech_hex27.cuh"
#include "fec_mech_hex8.cuh"

namespace fec {
namespace {

constexpr int MIX_THREADS = 192, MIX_CTAS_PER_SM = 3;
constexpr int MIX_HEX8_EPB = 8, MIX_TET4_EPB = 16, MIX_TET10_EPB = 3;  // tet10: 2 column chunks per row
constexpr int MIX_MAX_BLOCKS = MIXED_MAX_BLOCKS;

struct MixedBlocks {
  int n;
  int type[MIX_MAX_BLOCKS];
  unsigned tile_start[MIX_MAX_BLOCKS + 1];
  ElemArgs args[MIX_MAX_BLOCKS];
};

// One function per element type, not inlined into the kernel: each is register
// allocated on its own (as in its per-block kernel) instead of as one body.
template <class Model, bool R, bool K>
__device__ __noinline__ void tile_hex8(const ElemArgs& g, unsigned tile, int tid, unsigned char* sm) {
  hex8_df64_tile<Model, MIX_HEX8_EPB, R, K, false>(g, tile, tid % 24, tid / 24, sm);
}
template <class Model, bool R, bool K>
__device__ __noinline__ void tile_tet4(const ElemArgs& g, unsigned tile, int tid, unsigned char* sm) {
  mech_element_tile<6, Model, double, MIX_TET4_EPB, 1, R, K>(g, tile, tid % 12, tid / 12, sm);
}
template <class Model, bool R, bool K>
__device__ __noinline__ void tile_tet10(const ElemArgs& g, unsigned tile, int tid, unsigned char* sm) {
  // threads 180..191: slot ty = 3, idle
  mech_element_tile<7, Model, double, MIX_TET10_EPB, 2, R, K, MIX_THREADS>(g, tile, tid % 60, tid / 60, sm);
}
template <class Model, bool R, bool K>
__device__ __noinline__ void tile_hex27(const ElemArgs& g, unsigned tile, int tid, unsigned char* sm) {
  hex27_df64_tile<Model, R, K, MIX_THREADS>(g, tile, tid, sm);
}

template <class Model, bool R, bool K>
__device__ __forceinline__ void run_tile(int type, const ElemArgs& g, unsigned tile, int tid, unsigned char* sm) {
  switch (type) {
    case 1: tile_hex8<Model, R, K>(g, tile, tid, sm); break;
    case 6: tile_tet4<Model, R, K>(g, tile, tid, sm); break;
    case 7: tile_tet10<Model, R, K>(g, tile, tid, sm); break;
    default: tile_hex27<Model, R, K>(g, tile, tid, sm); break;
  }
}

template <class Model, bool R, bool K>
__global__ void __launch_bounds__(MIX_THREADS, MIX_CTAS_PER_SM)
    mixed_df64_kernel(const __grid_constant__ MixedBlocks m, unsigned* next_tile) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned s_item;
  const unsigned total = m.tile_start[m.n];
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(next_tile, 1u);
    __syncthreads();
    const unsigned item = s_item;
    if (item >= total) break;  // the same value in every thread of the CTA
    int b = 0;
    while (b + 1 < m.n && item >= m.tile_start[b + 1]) ++b;
    // the block's arguments are read in place from the (grid-constant) parameter block
    run_tile<Model, R, K>(m.type[b], m.args[b], item - m.tile_start[b], threadIdx.x, smem_raw);
    __syncthreads();  // the next tile reuses the shared memory and s_item
  }
}

template <class Model>
constexpr size_t mixed_smem(bool want_k) {
  const size_t a = Hex8Df64Smem<Model, MIX_HEX8_EPB>::BYTES;
  const size_t b = want_k ? mech_smem_bytes<6, Model, double, MIX_TET4_EPB, true>()
                          : mech_smem_bytes<6, Model, double, MIX_TET4_EPB, false>();
  const size_t c = want_k ? mech_smem_bytes<7, Model, double, MIX_TET10_EPB, true>()
                          : mech_smem_bytes<7, Model, double, MIX_TET10_EPB, false>();
  const size_t d = Hex27Df64Smem<Model>::BYTES;
  size_t m = a > b ? a : b;
  m = m > c ? m : c;
  return m > d ? m : d;
}

template <class Model, bool R, bool K>
cudaError_t go(const MixedBlocks& m, unsigned* counter, cudaStream_t s) {
  const size_t smem = mixed_smem<Model>(K);
  cudaError_t e;
  if ((e = ensure_smem<mixed_df64_kernel<Model, R, K>>(smem)) != cudaSuccess) return e;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned total = m.tile_start[m.n];
  const unsigned slots = unsigned(MIX_CTAS_PER_SM * sms);
  const unsigned grid = total < slots ? total : slots;
  if ((e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s)) != cudaSuccess) return e;
  mixed_df64_kernel<Model, R, K><<<grid, MIX_THREADS, smem, s>>>(m, counter);
  return cudaGetLastError();
}

template <class Model>
cudaError_t dispatch(bool want_r, bool want_k, const MixedBlocks& m, unsigned* counter, cudaStream_t s) {
  if (want_r && want_k) return go<Model, true, true>(m, counter, s);
  if (want_r) return go<Model, true, false>(m, counter, s);
  return go<Model, false, true>(m, counter, s);
}

}  // namespace

bool mixed_launch_supported(int physics, int nblocks, const int* elem_types) {
  if (physics != 2 && physics != 3) return false;
  if (nblocks < 1 || nblocks > MIX_MAX_BLOCKS) return false;
  for (int b = 0; b < nblocks; ++b) {
    const int t = elem_types[b];
    if (t != 1 && t != 6 && t != 7 && t != 8) return false;
  }
  return true;
}

cudaError_t launch_mech_mixed(int physics, int nblocks, const int* elem_types, const ElemArgs* args, bool want_r,
                              bool want_k, unsigned* tile_counter, cudaStream_t s, int* launches) {
  if (!mixed_launch_supported(physics, nblocks, elem_types)) return cudaErrorNotSupported;
  if (!tile_counter) return cudaErrorInvalidValue;
  if (!want_r && !want_k) return cudaSuccess;
  // work of one tile ~ elements x (element dofs)^2 x points: hex27 1 x 81^2 x 27,
  // hex8 8 x 24^2 x 8, tet10 3 x 30^2 x 5, tet4 16 x 12^2 x 1
  auto tile_work = [](int t) -> int64_t {
    return t == 8 ? 177147 : (t == 1 ? 36864 : (t == 7 ? 13500 : 2304));
  };
  int order[MIX_MAX_BLOCKS];
  for (int b = 0; b < nblocks; ++b) order[b] = b;
  for (int i = 1; i < nblocks; ++i)  // stable insertion sort, heaviest first
    for (int j = i; j > 0 && tile_work(elem_types[order[j]]) > tile_work(elem_types[order[j - 1]]); --j) {
      const int tmp = order[j];
      order[j] = order[j - 1];
      order[j - 1] = tmp;
    }
  MixedBlocks m{};
  m.n = nblocks;
  unsigned start = 0;
  for (int k = 0; k < nblocks; ++k) {
    const int b = order[k];
    const int t = elem_types[b];
    const int64_t per = t == 1 ? MIX_HEX8_EPB : (t == 6 ? MIX_TET4_EPB : (t == 7 ? MIX_TET10_EPB : 1));
    const int64_t tiles = (args[b].ne + per - 1) / per;
    if (tiles < 0 || int64_t(start) + tiles >= (int64_t(1) << 31)) return cudaErrorNotSupported;
    m.type[k] = t;
    m.args[k] = args[b];
    m.tile_start[k] = start;
    start += unsigned(tiles);
  }
  m.tile_start[nblocks] = start;
  for (int b = nblocks; b < MIX_MAX_BLOCKS; ++b) m.tile_start[b + 1] = start;
  if (start == 0) return cudaSuccess;
  ++*launches;
  return physics == 2 ? dispatch<NeoHookean>(want_r, want_k, m, tile_counter, s)
                      : dispatch<J2>(want_r, want_k, m, tile_counter, s);
}

}  // namespace fec
