// fec_closure_tc.cu -- the learned J2 closure on the 5th-generation tensor cores.
//
// A persistent CTA of 288 threads (eight epilogue warps and one warp that
// issues the MMAs) takes 16 hex8 elements (128 quadrature points, the M = 128 of
// one tcgen05 MMA) at a time:
//   A  element staging, isoparametric map and displacement gradient per point,
//      trial state; elastic points are completed exactly, plastic points write
//      their normalised input row to the first layer's operand tile;
//   B  the 14-64-64-64-64-13 SiLU network with its forward-mode Jacobian: per
//      point one activation row and six tangent rows (d/d e_tr of the six strain
//      inputs) go through every layer as one BF16 MMA each per K step, with FP32
//      accumulators in tensor memory.  The activation row uses a two-term BF16
//      split of activations and weights (hi*Whi + lo*Whi + hi*Wlo), which keeps
//      the stress near FP32 accuracy; tangent rows use one BF16 term.  Between
//      layers the eight epilogue warps read the accumulators back (tcgen05.ld),
//      apply bias, SiLU and SiLU' and write the next operand tiles;
//   C  per plastic point: stress and tangent from the outputs, the consistency
//      check, and the exact return map where the check fails.
// C of one tile (warps 0..3) runs concurrently with A of the next (warps 4..7).
// Each point's stress (Voigt) and 6x6 tangent go to a point table; the FP32 hex8
// element kernel (point-table model) then forms R_e and K_e from it.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>
#include "../../include/fec_gb300.h"
#include "fec_closure_physics.cuh"
#include "fec_closure_tc.h"
#include "fec_launch.h"
#include "fec_mech_hex8.cuh"
#include "fec_tc.cuh"

namespace fec {
namespace tcmlp {

// ---- parameter image (global memory, copied verbatim into shared memory) -------
constexpr uint32_t W0H = 0, W0L = 2048;                       // 64 x 16 BF16 each (inputs padded 14 -> 16)
__host__ __device__ constexpr uint32_t WH(int l) { return 4096 + uint32_t(l - 1) * 16384; }  // l = 1..3, 64 x 64
__host__ __device__ constexpr uint32_t WL(int l) { return WH(l) + 8192; }
constexpr uint32_t W4H = 53248, W4L = 55296;                  // 16 x 64 BF16 each (outputs padded 13 -> 16)
constexpr uint32_t F32 = 57344;                               // FP32 section
constexpr int FB = 0;                                         // biases of layers 0..3: 64 each
constexpr int FB4 = 256;                                      // output bias, 16
constexpr int FW0T = 272;                                     // [64][6] W0[o][j] / in_std[j]
constexpr int FIN_MEAN = 656, FIN_RSTD = 672, FOUT_MEAN = 688, FOUT_STD = 704;
constexpr int NF32 = 720;
constexpr uint32_t IMG_BYTES = F32 + NF32 * 4;                // 60,224
static_assert(IMG_BYTES % 16 == 0, "image copied in 16-byte words");

// ---- shared memory of the MLP stage ------------------------------------------------
constexpr uint32_t S_IMG = 0;
constexpr uint32_t S_ACT_H = 60416, S_ACT_L = S_ACT_H + 16384;  // 128 x 64 BF16 each
constexpr uint32_t S_TAN0 = S_ACT_L + 16384;                     // six 128 x 64 BF16 tangent tiles
__host__ __device__ constexpr uint32_t S_TAN(int j) { return S_TAN0 + uint32_t(j) * 16384; }
constexpr uint32_t S_X0_H = S_TAN0 + 5 * 16384, S_X0_L = S_X0_H + 4096;  // 128 x 16 input rows (alias tangent 5)
constexpr uint32_t S_BAR = S_TAN0 + 6 * 16384;                   // mbarriers: activation MMAs, tangent MMAs
constexpr uint32_t S_TSLOT = S_BAR + 16;                         // TMEM base address
constexpr uint32_t S_ABORT = S_BAR + 20;                         // set when an epilogue wait gave up
constexpr uint32_t S_USER = S_BAR + 128;                         // 191,616: caller's region
static_assert(S_IMG + IMG_BYTES <= S_ACT_H, "image overlaps the operand tiles");

constexpr int NEPI = 256;          // epilogue / point threads (warps 0..7)
constexpr int NTHR = NEPI + 32;    // + one warp that only issues MMAs (warp 8)
constexpr int CW = 64 * 128 / NEPI;  // hidden columns per thread in an epilogue (32)
constexpr uint32_t TMEM_COLS = 512;          // 7 accumulators x 64 columns
constexpr long long WAIT_BUDGET = 2000000000LL;  // SM clocks (about 1 s) before a wait gives up

// ---- host: pack FP32 parameters and normalisation into the image ---------------------
void put(std::vector<unsigned char>& img, uint32_t base, int r, int k, int K, __nv_bfloat16 v) {
  std::memcpy(&img[base + tc::op_offset(r, k & ~7, K) + (k & 7) * 2], &v, 2);
}
void put_split(std::vector<unsigned char>& img, uint32_t hi, uint32_t lo, int r, int k, int K, float w) {
  const __nv_bfloat16 h = __float2bfloat16_rn(w);
  put(img, hi, r, k, K, h);
  put(img, lo, r, k, K, __float2bfloat16_rn(w - __bfloat162float(h)));
}

}  // namespace tcmlp

std::vector<unsigned char> pack_mlp_image(const float* params, const float* norm) {
  using namespace tcmlp;
  std::vector<unsigned char> img(IMG_BYTES, 0);
  float* f = reinterpret_cast<float*>(img.data() + F32);
  const float* in_mean = norm;
  const float* in_std = norm + MLP_IN;
  const float* out_mean = norm + 2 * MLP_IN;
  const float* out_std = norm + 2 * MLP_IN + MLP_OUT;
  for (int l = 0; l < MLP_LAYERS; ++l) {
    const int nin = mlp_dim(l), nout = mlp_dim(l + 1);
    const float* W = params + mlp_w_off(l);
    const float* b = params + mlp_b_off(l);
    for (int o = 0; o < nout; ++o) {
      for (int i = 0; i < nin; ++i) {
        const float w = W[o * nin + i];
        if (l == 0) put_split(img, W0H, W0L, o, i, 16, w);
        else if (l < MLP_LAYERS - 1) put_split(img, WH(l), WL(l), o, i, 64, w);
        else put_split(img, W4H, W4L, o, i, 64, w);
      }
      f[(l < MLP_LAYERS - 1 ? FB + 64 * l : FB4) + o] = b[o];
    }
  }
  for (int o = 0; o < MLP_HID; ++o)
    for (int j = 0; j < 6; ++j) f[FW0T + o * 6 + j] = params[mlp_w_off(0) + o * MLP_IN + j] / in_std[j];
  for (int i = 0; i < MLP_IN; ++i) {
    f[FIN_MEAN + i] = in_mean[i];
    f[FIN_RSTD + i] = 1.0f / in_std[i];
  }
  for (int o = 0; o < MLP_OUT; ++o) {
    f[FOUT_MEAN + o] = out_mean[o];
    f[FOUT_STD + o] = out_std[o];
  }
  return img;
}

namespace tcmlp {

// ---- device: the MLP stage ------------------------------------------------------------
struct Ctx {
  unsigned char* sm;  // dynamic shared memory
  uint32_t s0;        // its shared-space address
  uint32_t tmem;      // TMEM base (lane 0, first column)
  uint64_t* bar_a;    // completes when a layer's activation-row MMAs are done
  uint64_t* bar_t;    // ... its tangent-row MMAs
  uint32_t phase_a, phase_t;
};

// The shared-space base address as a value the compiler cannot treat as loop
// invariant: the ~100 descriptors of a tile's MMAs are then formed just before
// each issue (a few integer operations) instead of being hoisted out of the tile
// loop and kept live -- which spilled them to local memory and made the single
// issuing thread wait on L2 for every MMA.
__device__ __forceinline__ uint32_t opaque(uint32_t v) {
  uint32_t r;
  asm volatile("mov.b32 %0, %1;" : "=r"(r) : "r"(v));
  return r;
}

// MMAs of layer l, issued by one thread.  Accumulator of row vector v at
// columns 64 v: v = 0 the activation row, v = 1 + j the tangent of input j.
// Activation rows: hi*Whi + lo*Whi + hi*Wlo; tangent rows: t*Whi.
__device__ __forceinline__ void issue_act(const Ctx& c, int l) {
  using namespace tc;
  const uint32_t s0 = opaque(c.s0);
  if (l == 0) {
    const uint32_t id = idesc_bf16(128, 64);
    const uint64_t xh = smem_desc(s0 + S_X0_H, 128, 256), xl = smem_desc(s0 + S_X0_L, 128, 256);
    const uint64_t wh = smem_desc(s0 + S_IMG + W0H, 128, 256), wl = smem_desc(s0 + S_IMG + W0L, 128, 256);
    mma_bf16(c.tmem, xh, wh, id, 0);
    mma_bf16(c.tmem, xl, wh, id, 1);
    mma_bf16(c.tmem, xh, wl, id, 1);
    return;
  }
  const bool out = l == MLP_LAYERS - 1;
  const uint32_t id = idesc_bf16(128, out ? 16 : 64);
  const uint32_t wH = S_IMG + (out ? W4H : WH(l)), wL = S_IMG + (out ? W4L : WL(l));
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const uint32_t ko = uint32_t(s) * 256;
    const uint64_t ah = smem_desc(s0 + S_ACT_H + ko, 128, 1024), al = smem_desc(s0 + S_ACT_L + ko, 128, 1024);
    const uint64_t bh = smem_desc(s0 + wH + ko, 128, 1024), bl = smem_desc(s0 + wL + ko, 128, 1024);
    mma_bf16(c.tmem, ah, bh, id, s > 0);
    mma_bf16(c.tmem, al, bh, id, 1);
    mma_bf16(c.tmem, ah, bl, id, 1);
  }
}
__device__ __forceinline__ void issue_tan(const Ctx& c, int l) {  // l >= 1
  using namespace tc;
  const uint32_t s0 = opaque(c.s0);
  const bool out = l == MLP_LAYERS - 1;
  const uint32_t id = idesc_bf16(128, out ? 16 : 64);
  const uint32_t wH = S_IMG + (out ? W4H : WH(l));
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const uint32_t ko = uint32_t(s) * 256;
    const uint64_t bh = smem_desc(s0 + wH + ko, 128, 1024);
#pragma unroll
    for (int j = 0; j < 6; ++j)
      mma_bf16(c.tmem + 64u * (1 + j), smem_desc(s0 + S_TAN(j) + ko, 128, 1024), bh, id, s > 0);
  }
}

// SiLU and its derivative with one exponential and one fast division.
__device__ __forceinline__ void silu_and_prime(float z, float& a, float& d) {
  const float s = __fdividef(1.0f, 1.0f + __expf(-z));
  a = z * s;
  d = s * (1.0f + z * (1.0f - s));
}

// Hidden layer l (0..3) epilogues, epilogue warps 0..7: warp w reads lanes 32 (w % 4) ..
// (points), columns 32 (w / 4) .. +31 of the layer's 64 outputs.  The
// activation part writes the next activation tiles and keeps SiLU' in d; the
// tangent part scales the tangent accumulators by it (layer 0: the input seeds).
__device__ __forceinline__ void epilogue_act(const Ctx& c, int l, float d[CW]) {
  using namespace tc;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qd = warp & 3, m = 32 * qd + lane, c0 = CW * (warp >> 2);
  const float* f = reinterpret_cast<const float*>(c.sm + S_IMG + F32);
  const uint32_t row = c.tmem + (uint32_t(32 * qd) << 16);
  float z[CW];
  tmem_ld32(row + c0, z);
#pragma unroll
  for (int i = 0; i < CW; ++i) silu_and_prime(z[i] + f[FB + 64 * l + c0 + i], z[i], d[i]);
#pragma unroll
  for (int k8 = 0; k8 < CW / 8; ++k8) store8_split(c.sm + S_ACT_H, c.sm + S_ACT_L, m, c0 + 8 * k8, 64, z + 8 * k8);
}
__device__ __forceinline__ void epilogue_tan(const Ctx& c, int l, const float d[CW]) {
  using namespace tc;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int qd = warp & 3, m = 32 * qd + lane, c0 = CW * (warp >> 2);
  const float* f = reinterpret_cast<const float*>(c.sm + S_IMG + F32);
  const uint32_t row = c.tmem + (uint32_t(32 * qd) << 16);
#pragma unroll 1
  for (int j = 0; j < 6; j += 2) {
    float t[2][CW];
    if (l == 0) {
#pragma unroll
      for (int i = 0; i < CW; ++i) {
        t[0][i] = d[i] * f[FW0T + (c0 + i) * 6 + j];
        t[1][i] = d[i] * f[FW0T + (c0 + i) * 6 + j + 1];
      }
    } else {
      tmem_ld32x2(row + 64u * (1 + j) + c0, row + 64u * (2 + j) + c0, t[0], t[1]);
#pragma unroll
      for (int i = 0; i < CW; ++i) {
        t[0][i] *= d[i];
        t[1][i] *= d[i];
      }
    }
#pragma unroll
    for (int k8 = 0; k8 < CW / 8; ++k8) {
      store8(c.sm + S_TAN(j), m, c0 + 8 * k8, 64, t[0] + 8 * k8);
      store8(c.sm + S_TAN(j + 1), m, c0 + 8 * k8, 64, t[1] + 8 * k8);
    }
  }
}

// Named barriers between the epilogue warps (arrive) and the issuer warp (sync):
// 1 = activation operand tiles (or the input rows) ready, 2 = tangent tiles
// ready; 3 = the epilogue warps among themselves.
__device__ __forceinline__ void named_arrive(int id, int n) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void epi_sync() { named_sync(3, NEPI); }

// Epilogue warps: operand tiles written by this thread visible to the tensor
// core, this thread's TMEM reads complete, then signal the issuer.  After an
// abort the epilogue warps wait for the issuer at each barrier instead of
// arriving ahead of it, so no barrier generation is overrun.
__device__ __forceinline__ void release_to_issuer(int id, bool ok) {
  tc::fence_async_smem();
  tc::tc_fence_before();
  if (ok)
    named_arrive(id, NTHR);
  else
    named_sync(id, NTHR);
}

__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t& phase) {
  const bool ok = tc::mbar_wait(bar, phase, WAIT_BUDGET);
  phase ^= 1u;
  return ok;
}

// The issuer warp's part of one tile: layer l's MMAs as soon as the epilogue
// warps release their operand tiles.  Issues nothing once the epilogue warps
// have flagged an abort, but keeps the barrier sequence.
__device__ void issue_tile(Ctx& c) {
  using namespace tc;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(c.sm + S_ABORT);
  const bool leader = (threadIdx.x & 31) == 0;
  named_sync(1, NTHR);  // input rows
  tc_fence_after();
  if (leader && !*abort_flag) {
    issue_act(c, 0);
    mma_commit(c.bar_a);
  }
  for (int l = 0; l < MLP_LAYERS - 1; ++l) {
    named_sync(1, NTHR);  // activation tiles of layer l
    tc_fence_after();
    if (leader && !*abort_flag) {
      issue_act(c, l + 1);
      mma_commit(c.bar_a);
    }
    named_sync(2, NTHR);  // tangent tiles of layer l
    tc_fence_after();
    if (leader && !*abort_flag) {
      issue_tan(c, l + 1);
      mma_commit(c.bar_t);
    }
  }
}

// The epilogue warps' part of one tile, after they wrote the input rows: the
// five layers, leaving the output layer's accumulators in TMEM.  Schedule per
// layer: the activation MMAs of layer l+1 run while the epilogue warps work
// through the tangent epilogue of layer l, the tangent MMAs of layer l+1 while
// they work through the activation epilogue of layer l+1, and the issuer warp
// issues in parallel with both.  `ok` goes (uniformly) false when a wait gives
// up; the barrier sequence is kept so that the issuer warp never blocks.
// `mid` runs once on every epilogue thread after layer 0 (a point where the
// caller can issue background work).
struct NoMid {
  __device__ void operator()() const {}
};
template <class Mid = NoMid>
__device__ void epilogue_tile(Ctx& c, bool& ok, const Mid& mid = Mid()) {
  using namespace tc;
  int* abort_flag = reinterpret_cast<int*>(c.sm + S_ABORT);
  release_to_issuer(1, ok);
  for (int l = 0; l < MLP_LAYERS - 1; ++l) {
    if (ok) {
      const bool w = wait_bar(c.bar_a, c.phase_a);
      if (!w) *abort_flag = 1;
    }
    epi_sync();
    ok = ok && !*reinterpret_cast<volatile int*>(abort_flag);
    tc_fence_after();
    float d[CW];
    if (ok) epilogue_act(c, l, d);
    release_to_issuer(1, ok);
    if (l > 0) {
      if (ok) {
        const bool w = wait_bar(c.bar_t, c.phase_t);
        if (!w) *abort_flag = 1;
      }
      epi_sync();
      ok = ok && !*reinterpret_cast<volatile int*>(abort_flag);
      tc_fence_after();
    }
    if (ok) epilogue_tan(c, l, d);
    release_to_issuer(2, ok);
    if (l == 0) mid();
  }
  if (ok) {
    const bool wa = wait_bar(c.bar_a, c.phase_a);
    const bool wt = wait_bar(c.bar_t, c.phase_t);
    if (!(wa && wt)) *abort_flag = 1;
  }
  epi_sync();
  ok = ok && !*reinterpret_cast<volatile int*>(abort_flag);
  tc_fence_after();
}

// Output layer epilogue for point m = threadIdx.x (warps 0..3 only): outputs y in
// physical units and the Jacobian of the six stress outputs w.r.t. e_tr.
__device__ __forceinline__ void epilogue_output(const Ctx& c, float y[MLP_OUT], float Js[6][6]) {
  using namespace tc;
  const int warp = threadIdx.x >> 5;
  const float* f = reinterpret_cast<const float*>(c.sm + S_IMG + F32);
  const uint32_t row = c.tmem + (uint32_t(32 * warp) << 16);
  float z[16];
  tmem_ld16(row, z);
#pragma unroll
  for (int o = 0; o < MLP_OUT; ++o) y[o] = (z[o] + f[FB4 + o]) * f[FOUT_STD + o] + f[FOUT_MEAN + o];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    tmem_ld16(row + 64u * (1 + j), z);
#pragma unroll
    for (int o = 0; o < 6; ++o) Js[o][j] = z[o] * f[FOUT_STD + o];
  }
}

// Normalised input row of point m (x in physical units; nullptr: a zero row).
__device__ __forceinline__ void write_input_row(const Ctx& c, int m, const float* x) {
  const float* f = reinterpret_cast<const float*>(c.sm + S_IMG + F32);
  float v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = (x && i < MLP_IN) ? (x[i] - f[FIN_MEAN + i]) * f[FIN_RSTD + i] : 0.f;
  tc::store8_split(c.sm + S_X0_H, c.sm + S_X0_L, m, 0, 16, v);
  tc::store8_split(c.sm + S_X0_H, c.sm + S_X0_L, m, 8, 16, v + 8);
}

// CTA prologue: image -> shared memory, mbarrier, TMEM.
__device__ void setup(Ctx& c, unsigned char* sm, const unsigned char* image) {
  using namespace tc;
  c.sm = sm;
  c.s0 = smem_u32(sm);
  c.bar_a = reinterpret_cast<uint64_t*>(sm + S_BAR);
  c.bar_t = reinterpret_cast<uint64_t*>(sm + S_BAR + 8);
  c.phase_a = c.phase_t = 0;
  const uint4* src = reinterpret_cast<const uint4*>(image);
  uint4* dst = reinterpret_cast<uint4*>(sm + S_IMG);
  for (int i = threadIdx.x; i < int(IMG_BYTES / 16); i += blockDim.x) dst[i] = src[i];
  if (threadIdx.x == 0) {
    *reinterpret_cast<int*>(sm + S_ABORT) = 0;
    mbar_init(c.bar_a, 1);
    mbar_init(c.bar_t, 1);
    mbar_fence_init();
  }
  if (threadIdx.x < 32) tmem_alloc(reinterpret_cast<uint32_t*>(sm + S_TSLOT), TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  c.tmem = *reinterpret_cast<volatile uint32_t*>(sm + S_TSLOT);
}

// CTA epilogue: after a timeout, give the MMAs in flight one more bounded wait;
// then release TMEM.
__device__ void teardown(Ctx& c, bool failed, int* err) {
  using namespace tc;
  if (failed) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    mbar_wait(c.bar_a, c.phase_a ^ 1u, WAIT_BUDGET);
    mbar_wait(c.bar_t, c.phase_t ^ 1u, WAIT_BUDGET);
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    tmem_dealloc(c.tmem, TMEM_COLS);
  }
}

// ---- standalone evaluation of the network on rows of X -----------------------------
__global__ void __launch_bounds__(NTHR, 1)
    mlp_eval_tc_kernel(const unsigned char* image, const float* X, int64_t n, float* Y, float* Jac, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  Ctx c;
  setup(c, sm, image);
  bool ok = true;
  const bool issuer = threadIdx.x >= NEPI;
  const int64_t tiles = (n + 127) / 128;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    if (issuer) {
      issue_tile(c);
    } else {
      const int64_t r = t * 128 + threadIdx.x;
      if (threadIdx.x < 128) {
        float x[MLP_IN];
        if (r < n)
          for (int i = 0; i < MLP_IN; ++i) x[i] = X[r * MLP_IN + i];
        write_input_row(c, threadIdx.x, r < n ? x : nullptr);
      }
      epilogue_tile(c, ok);
      if (ok && threadIdx.x < 128) {
        float y[MLP_OUT], Js[6][6];
        epilogue_output(c, y, Js);
        if (r < n) {
          for (int o = 0; o < MLP_OUT; ++o) Y[r * MLP_OUT + o] = y[o];
          for (int o = 0; o < 6; ++o)
            for (int j = 0; j < 6; ++j) Jac[r * 36 + o * 6 + j] = Js[o][j];
        }
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (*reinterpret_cast<volatile int*>(sm + S_ABORT)) break;
  }
  teardown(c, *reinterpret_cast<volatile int*>(sm + S_ABORT) != 0, err);
}

// ---- the closure over hex8 elements: point table and state ----------------------------
constexpr int EPT = 16;  // elements per tile (x 8 points = 128)
constexpr uint32_t U_REF = S_USER;                         // 264 doubles
constexpr uint32_t U_REFF = U_REF + 264 * 8;               // 264 floats
constexpr uint32_t U_X = U_REFF + 1072;                    // EPT x 24 doubles (prefetched)
constexpr uint32_t U_UD = U_X + EPT * 24 * 8;              // EPT x 24 doubles (prefetched)
constexpr uint32_t U_ST = U_UD + EPT * 24 * 8;             // 2 x 128 x 7 doubles: state_old (prefetched, parity)
constexpr uint32_t U_XD = U_ST + 2 * 128 * 7 * 8;          // EPT x 24 floats
constexpr uint32_t U_U = U_XD + EPT * 24 * 4;              // EPT x 24 floats
constexpr uint32_t U_GU = U_U + EPT * 24 * 4;              // 2 x 128 x 9 floats (tile parity)
constexpr uint32_t U_FLAG = U_GU + 2 * 128 * 9 * 4;        // 2 x 128 ints
constexpr uint32_t U_CONN = U_FLAG + 2 * 128 * 4;          // 128 ints (prefetched)
constexpr uint32_t POINTS_SMEM = U_CONN + 128 * 4;
constexpr int PREP_BAR = 4;                                // named barrier of the preparing warps 4..7
static_assert(POINTS_SMEM <= 227 * 1024, "closure kernel shared memory");
static_assert(RefLayout<1>::SIZE == 264, "hex8 reference tables");

__device__ __forceinline__ void write_row(float* table, int64_t p, const float* P9, const float* C36) {
  float4* dst = reinterpret_cast<float4*>(table + p * POINT_TABLE_STRIDE);
  const int ii[6] = {0, 1, 2, 1, 0, 0}, jj[6] = {0, 1, 2, 2, 2, 1};
  float v[POINT_TABLE_STRIDE];
#pragma unroll
  for (int m = 0; m < 6; ++m) v[m] = P9[ii[m] * 3 + jj[m]];
#pragma unroll
  for (int m = 0; m < 36; ++m) v[6 + m] = C36[m];
  v[42] = v[43] = 0.f;
#pragma unroll
  for (int k = 0; k < POINT_TABLE_STRIDE / 4; ++k) dst[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
}

// Background staging of tile t by warps 4..7 (m = 0..127), in two steps so that
// their latency hides under the previous tile's network: the connectivity (at
// the start of the previous tile), then -- it has landed by the end of that
// tile's first layer -- the coordinates, displacements and old state.
__device__ void prefetch_conn(const ElemArgs& g, const Ctx& c, int64_t t, int m) {
  int* s_conn = reinterpret_cast<int*>(c.sm + U_CONN);
  const int64_t e = t * EPT + m / 8;
  if (e < g.ne)
    tc::cp_async4(&s_conn[m], &g.conn[e * 8 + (m & 7)]);
  else
    s_conn[m] = 0;
  tc::cp_async_commit();
}
__device__ void prefetch_data(const ElemArgs& g, const Ctx& c, int64_t t, int buf, int m) {
  unsigned char* sm = c.sm;
  const int* s_conn = reinterpret_cast<const int*>(sm + U_CONN);
  double* s_x = reinterpret_cast<double*>(sm + U_X);
  double* s_ud = reinterpret_cast<double*>(sm + U_UD);
  double* s_st = reinterpret_cast<double*>(sm + U_ST) + buf * 128 * 7;
  tc::cp_async_wait_all();
  named_sync(PREP_BAR, 128);
  const int64_t e0 = t * EPT;
  for (int i = m; i < EPT * 24; i += 128) {
    const int el = i / 24, k = i % 24, a = k / 3, d = k % 3;
    if (e0 + el < g.ne) {
      const int64_t dof = int64_t(s_conn[el * 8 + a]) * 3 + d;
      tc::cp_async8(&s_x[i], &g.coords[dof]);
      tc::cp_async8(&s_ud[i], &g.U[dof]);
    }
  }
  const int64_t left = (g.ne - e0) * 8;
  const int nst = 7 * int(left < 128 ? left : 128);
  const double* so = g.state_old + e0 * 8 * 7;
  for (int j = m; j < nst; j += 128) tc::cp_async8(&s_st[j], &so[j]);
  tc::cp_async_commit();
}

// Phase A of tile t on warps 4..7 (m = point of the tile), from the staged
// data: map and displacement gradient, trial state; elastic points are
// completed exactly, plastic points write their input row (others a zero row).
// Flags and grad u go to the buffer of the tile's parity.
__device__ void prep_tile(const ElemArgs& g, const TcClosure& cl, const Ctx& c, int64_t t, int buf, int m) {
  unsigned char* sm = c.sm;
  const double* s_ref = reinterpret_cast<const double*>(sm + U_REF);
  const float* s_reff = reinterpret_cast<const float*>(sm + U_REFF);
  const double* s_x = reinterpret_cast<const double*>(sm + U_X);
  const double* s_ud = reinterpret_cast<const double*>(sm + U_UD);
  const double* s_st = reinterpret_cast<const double*>(sm + U_ST) + buf * 128 * 7;
  float* s_xd = reinterpret_cast<float*>(sm + U_XD);
  float* s_u = reinterpret_cast<float*>(sm + U_U);
  float* s_gu = reinterpret_cast<float*>(sm + U_GU) + buf * 128 * 9;
  int* s_flag = reinterpret_cast<int*>(sm + U_FLAG) + buf * 128;
  const int64_t e0 = t * EPT;
  tc::cp_async_wait_all();
  named_sync(PREP_BAR, 128);
  for (int i = m; i < EPT * 24; i += 128) {
    const int el = i / 24, d = i % 3;
    if (e0 + el < g.ne) {
      s_xd[i] = float(s_x[i] - s_x[el * 24 + d]);
      s_u[i] = float(s_ud[i]);
    }
  }
  named_sync(PREP_BAR, 128);
  const int el = m / 8, q = m & 7;
  const int64_t e = e0 + el, p = e * 8 + q;
  int flag = -1;  // -1: no element, 0: elastic (done), 1: plastic
  float x[MLP_IN];
  if (e < g.ne) {
    float dNX[24];
    map_hex8_mixed(s_ref, s_reff, q, s_x + el * 24, s_xd + el * 24, dNX);
    float gu[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        float sum = 0.f;
#pragma unroll
        for (int a = 0; a < 8; ++a) sum = fmaf(s_u[el * 24 + a * 3 + i], dNX[a * 3 + j], sum);
        gu[i][j] = sum;
        s_gu[m * 9 + i * 3 + j] = sum;
      }
    const double* so = s_st + m * 7;
    double* sn = g.state_new ? g.state_new + p * 7 : nullptr;
    float etr[6];
    if (J2MLP::trial(g.props, gu, so, etr, x)) {
      flag = 1;
    } else {
      float P9[9], C36[36];
      J2MLP::exact(g.props, gu, 1.0f, so, sn, P9, C36);
      write_row(cl.table, p, P9, C36);
      flag = 0;
    }
  }
  s_flag[m] = flag;
  write_input_row(c, m, flag == 1 ? x : nullptr);
  named_sync(PREP_BAR, 128);  // the staged data is free for the next tile
}

// Phase C of tile t on warps 0..3 (m = point of the tile): plastic points from
// the network's outputs, with the consistency check and the exact fallback.
// Each warp's 32 table rows are staged in shared memory (a tangent tile, idle
// between networks) and leave as contiguous 128-byte segments.
__device__ void complete_tile(const ElemArgs& g, const TcClosure& cl, const Ctx& c, int64_t t, int buf, int m) {
  const float* s_gu = reinterpret_cast<const float*>(c.sm + U_GU) + buf * 128 * 9;
  const int* s_flag = reinterpret_cast<const int*>(c.sm + U_FLAG) + buf * 128;
  const double* s_st = reinterpret_cast<const double*>(c.sm + U_ST) + buf * 128 * 7;
  float* stage = reinterpret_cast<float*>(c.sm + S_TAN(0)) + (m >> 5) * (32 * POINT_TABLE_STRIDE);
  float y[MLP_OUT], Js[6][6];
  epilogue_output(c, y, Js);
  const int plastic = s_flag[m] == 1;
  int fell_back = 0;
  if (plastic) {
    const int64_t p = t * 128 + m;
    const double* so = s_st + m * 7;
    double* sn = g.state_new ? g.state_new + p * 7 : nullptr;
    float gu[3][3];
#pragma unroll
    for (int i = 0; i < 9; ++i) gu[i / 3][i % 3] = s_gu[m * 9 + i];
    float etr[6];
    float x[MLP_IN];
    J2MLP::trial(g.props, gu, so, etr, x);
    float P9[9], C36[36];
    if (!J2MLP::finish(g.props, etr, cl.tol, y, Js, 1.0f, so, sn, P9, C36)) {
      fell_back = 1;
      J2MLP::exact(g.props, gu, 1.0f, so, sn, P9, C36);
    }
    float* row = stage + (m & 31) * POINT_TABLE_STRIDE;
    const int ii[6] = {0, 1, 2, 1, 0, 0}, jj[6] = {0, 1, 2, 2, 2, 1};
#pragma unroll
    for (int k = 0; k < 6; ++k) row[k] = P9[ii[k] * 3 + jj[k]];
#pragma unroll
    for (int k = 0; k < 36; ++k) row[6 + k] = C36[k];
    row[42] = row[43] = 0.f;
  }
  const unsigned pmask = __ballot_sync(0xffffffffu, plastic);
  const unsigned np = __popc(pmask);
  const unsigned nf = __popc(__ballot_sync(0xffffffffu, fell_back));
  if (np) {
    __syncwarp();
    const int lane = m & 31;
    float* dst = cl.table + (t * 128 + (m & ~31)) * POINT_TABLE_STRIDE;
    for (int f = lane; f < 32 * POINT_TABLE_STRIDE; f += 32)
      if ((pmask >> (f / POINT_TABLE_STRIDE)) & 1u) dst[f] = stage[f];
  }
  if ((m & 31) == 0 && np) {
    atomicAdd(&cl.counters[0], (unsigned long long)np);
    if (nf) atomicAdd(&cl.counters[1], (unsigned long long)nf);
  }
}

// Tiles of 16 elements.  Per tile the network runs on all eight epilogue warps
// (B); after it, warps 0..3 complete the tile's points (C) while warps 4..7
// already prepare the CTA's next tile (A), into the other parity's buffers and
// the input rows, which the tile's last MMAs no longer read.  The next tile's
// inputs are copied in the background during the current tile's network.
__global__ void __launch_bounds__(NTHR, 1) j2mlp_points_tc_kernel(ElemArgs g, TcClosure cl) {
  extern __shared__ __align__(1024) unsigned char sm[];
  Ctx c;
  setup(c, sm, cl.image);
  double* s_ref = reinterpret_cast<double*>(sm + U_REF);
  float* s_reff = reinterpret_cast<float*>(sm + U_REFF);
  const int tid = threadIdx.x;
  for (int i = tid; i < RefLayout<1>::SIZE; i += NTHR) {
    s_ref[i] = g.ref[i];
    s_reff[i] = float(g.ref[i]);
  }
  __syncthreads();
  bool ok = true;
  const bool issuer = tid >= NEPI;
  const int64_t tiles = (g.ne + EPT - 1) / EPT;
  int64_t t = blockIdx.x;
  const bool preparer = tid >= 128 && tid < NEPI;
  if (preparer && t < tiles) {
    prefetch_conn(g, c, t, tid - 128);
    prefetch_data(g, c, t, 0, tid - 128);
    prep_tile(g, cl, c, t, 0, tid - 128);
  }
  for (int it = 0; t < tiles; t += gridDim.x, ++it) {
    const int64_t tn = t + gridDim.x;
    const bool next = tn < tiles;
    if (issuer) {
      issue_tile(c);
    } else {
      if (preparer && next) prefetch_conn(g, c, tn, tid - 128);
      epilogue_tile(c, ok, [&] {
        if (preparer && next) prefetch_data(g, c, tn, (it + 1) & 1, tid - 128);
      });
      if (tid < 128) {
        if (ok) complete_tile(g, cl, c, t, it & 1, tid);
      } else if (next) {
        prep_tile(g, cl, c, tn, (it + 1) & 1, tid - 128);
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (*reinterpret_cast<volatile int*>(sm + S_ABORT)) break;
  }
  teardown(c, *reinterpret_cast<volatile int*>(sm + S_ABORT) != 0, reinterpret_cast<int*>(&cl.counters[2]));
}

// Point-table model for the FP32 hex8 element kernel: stress and tangent read
// from the table the closure kernel wrote (unscaled), scaled by JxW here.
struct J2Table {
  static constexpr bool USES_CLOSURE = false;
  static constexpr bool USES_TABLE = true;
  static constexpr int NS = 0;
  static constexpr int SCR = 36;
  template <typename Real>
  __device__ static void point_table(const void* table, int64_t p, Real jxw, Real* P9, Real* scr) {
    const float4* src = reinterpret_cast<const float4*>(static_cast<const float*>(table) + p * POINT_TABLE_STRIDE);
    float v[POINT_TABLE_STRIDE];
#pragma unroll
    for (int k = 0; k < POINT_TABLE_STRIDE / 4; ++k) {
      const float4 w = __ldg(src + k);
      v[4 * k] = w.x;
      v[4 * k + 1] = w.y;
      v[4 * k + 2] = w.z;
      v[4 * k + 3] = w.w;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P9[i * 3 + j] = jxw * v[voigt(i, j)];
#pragma unroll
    for (int m = 0; m < 36; ++m) scr[m] = jxw * v[6 + m];
  }
  template <typename Real>
  __device__ static Real aentry(const Real* scr, int i, int J, int k, int L) {
    return J2MLP::aentry(scr, i, J, k, L);
  }
  template <typename Real>
  __device__ static void point(const double*, Real (*)[3], Real, const double*, double*, Real*, Real*) {}
};

int sm_count() {
  static int count[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!count[dev]) cudaDeviceGetAttribute(&count[dev], cudaDevAttrMultiProcessorCount, dev);
  return count[dev] > 0 ? count[dev] : 148;
}

}  // namespace tcmlp

cudaError_t launch_j2mlp_points_tc(const ElemArgs& a, const TcClosure& cl, cudaStream_t s, int* launches) {
  using namespace tcmlp;
  if (a.ne <= 0) return cudaSuccess;
  cudaError_t e = ensure_smem<j2mlp_points_tc_kernel>(POINTS_SMEM);
  if (e != cudaSuccess) return e;
  const int64_t tiles = (a.ne + EPT - 1) / EPT;
  const unsigned grid = unsigned(tiles < sm_count() ? tiles : sm_count());
  j2mlp_points_tc_kernel<<<grid, NTHR, POINTS_SMEM, s>>>(a, cl);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_point_table_hex8(bool want_r, bool want_k, const ElemArgs& a, const float* table, cudaStream_t s,
                                    int* launches) {
  using namespace tcmlp;
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ElemArgs b = a;
  b.closure = table;
  constexpr int EPB = 16;
  const dim3 block(12, EPB), egrid(unsigned((a.ne + EPB - 1) / EPB));
  constexpr size_t smem = Hex8Smem<J2Table, float, EPB>::BYTES;
  cudaError_t e;
  ++*launches;
  if (want_r && want_k) {
    if ((e = ensure_smem<mech_hex8_rows2_kernel<J2Table, EPB, true, true>>(smem)) != cudaSuccess) return e;
    mech_hex8_rows2_kernel<J2Table, EPB, true, true><<<egrid, block, smem, s>>>(b);
  } else if (want_r) {
    if ((e = ensure_smem<mech_hex8_rows2_kernel<J2Table, EPB, true, false>>(smem)) != cudaSuccess) return e;
    mech_hex8_rows2_kernel<J2Table, EPB, true, false><<<egrid, block, smem, s>>>(b);
  } else {
    if ((e = ensure_smem<mech_hex8_rows2_kernel<J2Table, EPB, false, true>>(smem)) != cudaSuccess) return e;
    mech_hex8_rows2_kernel<J2Table, EPB, false, true><<<egrid, block, smem, s>>>(b);
  }
  return cudaGetLastError();
}

}  // namespace fec

extern "C" {

int fec_mlp_eval_tc(const float* params, const float* normalisation, const float* X_dev, int64_t n, float* Y_dev,
                    float* jac_dev, void* stream) {
  using namespace fec::tcmlp;
  if (!params || !normalisation || n < 0 || (n > 0 && (!X_dev || !Y_dev || !jac_dev))) return FEC_ERR_ARG;
  if (n == 0) return FEC_OK;
  const std::vector<unsigned char> img = fec::pack_mlp_image(params, normalisation);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* d_img = nullptr;
  int* d_err = nullptr;
  if (cudaMalloc(&d_img, img.size()) != cudaSuccess) return FEC_ERR_CUDA;
  if (cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) {
    cudaFree(d_img);
    return FEC_ERR_CUDA;
  }
  int status = FEC_OK, h_err = 0;
  if (cudaMemcpyAsync(d_img, img.data(), img.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemsetAsync(d_err, 0, sizeof(int), s) != cudaSuccess ||
      fec::ensure_smem<mlp_eval_tc_kernel>(S_USER) != cudaSuccess) {
    status = FEC_ERR_CUDA;
  } else {
    const int64_t tiles = (n + 127) / 128;
    const unsigned grid = unsigned(tiles < sm_count() ? tiles : sm_count());
    mlp_eval_tc_kernel<<<grid, NTHR, S_USER, s>>>(static_cast<const unsigned char*>(d_img), X_dev, n, Y_dev,
                                                  jac_dev, d_err);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      status = FEC_ERR_CUDA;
    else if (h_err)
      status = FEC_ERR_DEVICE;
  }
  cudaFree(d_img);
  cudaFree(d_err);
  return status;
}

}  // extern "C"
