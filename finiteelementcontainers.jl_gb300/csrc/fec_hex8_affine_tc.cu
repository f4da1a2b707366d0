// fec_hex8_affine_tc.cu -- FP64-accurate hex8 element stiffness on the tensor
// cores for blocks whose elements are translates of one another (structured
// meshes), by exact integer slicing of both operands (the Ozaki scheme: Ozaki,
// Ogita, Oishi and Rump, Numer. Algorithms 59 (2012) 95-118, restated here for
// BF16 digits and FP32 accumulation).
//
// The tangent of element e is (src/Formulations.jl:462-576)
//     K_(a,i),(b,k) = sum_q sum_(J,L) dNX_qaJ * JxW A_q,iJkL * dNX_qbL .
// With every element a translate of the first, dNX_q and JxW_q are the same for
// all elements, so with r = (q, J, L) (72 values) and the node pair n = (a, b),
// a <= b (36 pairs: the rest follow from K = K^T),
//     D[(e, i, k), n] = sum_r A_e[(e, i, k), r] * W[n, r],   W[n, r] = dNX_qaJ dNX_qbL,
// one GEMM over all elements with a constant right operand.  Each A row (one
// element, scaled by a power of two 2^tau_e over the element's largest entry)
// and each W row (2^sigma_n) is written as seven signed 8-bit digits,
//     x = 2^tau * sum_t d_t 2^(-7-8t),  |d_t| <= 256,
// every digit exact in BF16.  A digit product is an integer below 2^16 and a
// 72-term dot product of digits below 2^23, so the sums over r of all digit
// pairs with s + t = L (at most seven pairs, each with |d| <= 256 in one digit
// position per value at most) stay below 2^24: each level L = 0..6 accumulates
// exactly in its own FP32 TMEM accumulator.  Levels above 6 are dropped
// (contributions below 2^-56 of the scales); the epilogue sums the seven levels
// in double-float and scales by 2^(tau_e + sigma_n - 14).
//
// One persistent CTA per SM, tiles of 12 elements.  MMA row m = 32 w + 9 j + ik
// holds (element 3 w + j, ik = 3 i + k): every element's nine rows lie in one
// warp's TMEM lanes, lanes 27-31 of each warp are padding rows.
//   warps 0-2   FP64 point phase (displacement gradient, constitutive update),
//               one thread per quadrature point, into a staging area;
//   warps 3-8   tangent entries (45 unique per point, double-float), parked in
//               TMEM, then (once the previous tile's MMAs read the slices) their
//               digits into the seven A slices;
//   warp 9      the residual R = sum_q dNX P in double-float;
//   warps 10-13 the epilogue: TMEM -> double-float values (row (e, i, k) holds
//               K_(a,i),(b,k) for a <= b), stored as they leave tensor memory:
//               the symmetric half (KE_PAIRS, entry 9n + 3i + k of pair n), or
//               each value at its two places in the node rows of the whole K_e;
//   warp 14     issues the tile's 50 MMAs (10 groups of digit pairs x 5 K steps).
// The A slices are rewritten as soon as the MMAs that read them completed; the
// next MMAs wait only for the epilogue's reads of the accumulators.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>

#include "fec_df64.cuh"
#include "fec_kernels.cuh"
#include "fec_launch.h"
#include "fec_tc.cuh"

namespace fec {
namespace aff {

constexpr int EPT = 12;              // elements per tile (three per 32-row quarter)
constexpr int NQ = 8;
constexpr int NPT = EPT * NQ;        // quadrature points per tile (96)
constexpr int KR = 72, KP = 80;      // reduction length r = (q, J, L), padded to 5 K steps
constexpr int NPAIR = 36, NPAD = 48; // node pairs a <= b, padded N
constexpr int ND = 7;                // digits per operand
constexpr int NLEV = 7;              // accumulated levels s + t = 0..6
constexpr int SBO = KP * 16;         // bytes between 8-row groups of an operand tile
constexpr int A_SLICE = 128 * KP * 2;
constexpr int W_SLICE = NPAD * KP * 2;
// table built on the host (hex8_affine_table): W digits, sigma, dNX, JxW
constexpr int T_W = 0;
constexpr int T_SIG = ND * W_SLICE;
constexpr int T_G = T_SIG + NPAD * 4;
constexpr int T_JXW = T_G + NQ * 24 * 8;
constexpr int T_BYTES = T_JXW + NQ * 8;
static_assert(T_BYTES % 16 == 0 && T_G % 8 == 0, "table layout");
constexpr int TMEM_COLS = 512;
constexpr int TM_ENT = NLEV * NPAD;  // 2 x 48 columns after the accumulators: the slicers' scaled tangent entries (hi, lo)
static_assert(TM_ENT + 2 * 48 <= TMEM_COLS, "tensor memory columns");
constexpr long long WAIT_BUDGET = 2000000000LL;

constexpr int PROD_W = 3, SL_W = 6, R_W = 1, EP_W = 4, MMA_W = 1;
constexpr int NTHR = 32 * (PROD_W + SL_W + R_W + EP_W + MMA_W);
constexpr int T_SL = 32 * PROD_W, T_R = T_SL + 32 * SL_W, T_EP = T_R + 32 * R_W, T_MMA = T_EP + 32 * EP_W;
constexpr int NSL = 32 * SL_W;
static_assert(32 * PROD_W == NPT && NSL == 2 * NPT && (T_EP / 32) % 4 == 2, "roles");
// named barriers (0 is __syncthreads)
constexpr int BAR_FULL = 1;   // producers arrive, slicers + residual warp sync
constexpr int BAR_EMPTY = 2;  // slicers + residual warp arrive, producers sync
constexpr int N_FULL = 32 * (PROD_W + SL_W + R_W);

// The MMAs of a tile: A slice t against W slices s0 .. s0+ns-1 at once (consecutive
// W slices are consecutive 48-row blocks, one N = 48 ns operand), accumulating
// into levels s0+t .. s0+t+ns-1 (consecutive 48-column blocks).  Every pair
// s + t <= 6 once; the t = 0 groups write each level first.
constexpr int NGROUP = 10;
__device__ __constant__ int8_t kGroups[NGROUP][3] = {{0, 0, 4}, {0, 4, 3}, {1, 0, 4}, {1, 4, 2}, {2, 0, 4},
                                                      {2, 4, 1}, {3, 0, 4}, {4, 0, 3}, {5, 0, 2}, {6, 0, 1}};

// MMA row of (element el of the tile, ik = 3 i + k)
__host__ __device__ __forceinline__ int row_of(int el, int ik) { return 32 * (el / 3) + 9 * (el % 3) + ik; }

template <class Model>
struct Layout {
  static constexpr int W = 0;
  static constexpr int A = W + ND * W_SLICE;
  static constexpr int P = A + ND * A_SLICE;                      // float2 [96][9]
  static constexpr int SCR = P + NPT * 9 * 8;                     // float2 [96][SCR2]
  static constexpr int G = (SCR + NPT * Model::SCR2 * 8 + 15) / 16 * 16;  // double [8][24]
  static constexpr int G2 = G + NQ * 24 * 8;                      // float2 [8][24]
  static constexpr int JXW = G2 + NQ * 24 * 8;                    // double [8]
  static constexpr int SIG = JXW + NQ * 8;                        // int [48]
  static constexpr int TAU = SIG + NPAD * 4;                      // int [2][12]: per tile parity
  static constexpr int TAUST = TAU + 2 * 16 * 4;                  // int [12]: the staged tile's scales
  static constexpr int CODE = TAUST + 16 * 4;                     // uint32 [45] entry codes (+pad)
  static constexpr int BAR = (CODE + 48 * 4 + 15) / 16 * 16;      // mbarriers: slices, MMAs, TMEM read
  static constexpr int TSLOT = BAR + 32;
  static constexpr int SMEM = TSLOT + 16;
  static_assert(SMEM <= 232448, "shared memory");
};

__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void named_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}
// 2^k as a float for k in [-126, 127]
__device__ __forceinline__ float pow2f(int k) { return __uint_as_float(uint32_t(k + 127) << 23); }

// byte offset of element (row, col) in a K-major operand tile with K = 80
__host__ __device__ __forceinline__ uint32_t op_off(int row, int col) {
  return uint32_t(row >> 3) * SBO + uint32_t(col >> 3) * 128 + uint32_t(row & 7) * 16 + uint32_t(col & 7) * 2;
}
// Seven 4-column loads (the seven levels of one column chunk) under one wait.
__device__ __forceinline__ void tmem_ld4x7(uint32_t taddr, float (*v)[4]) {
  uint32_t r[28];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%28];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%4, %5, %6, %7}, [%29];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%8, %9, %10, %11}, [%30];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%12, %13, %14, %15}, [%31];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16, %17, %18, %19}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%20, %21, %22, %23}, [%33];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%24, %25, %26, %27}, [%34];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27])
      : "r"(taddr), "r"(taddr + 48u), "r"(taddr + 96u), "r"(taddr + 144u), "r"(taddr + 192u), "r"(taddr + 240u),
        "r"(taddr + 288u)
      : "memory");
#pragma unroll
  for (int L = 0; L < NLEV; ++L)
#pragma unroll
    for (int j = 0; j < 4; ++j) v[L][j] = __uint_as_float(r[L * 4 + j]);
}

__device__ __forceinline__ void tmem_st2(uint32_t taddr, float a, float b) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};" ::"r"(taddr), "r"(__float_as_uint(a)),
               "r"(__float_as_uint(b))
               : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }


// Point phase of quadrature point q of element e (FP64): the eight lanes of an
// element (consecutive, aligned to 8) each load one node's displacement and
// share it; gu = sum_a u_a (x) dNX_qa; the constitutive update.  Every lane of
// the warp calls it (the shuffles); `live` lanes get P9 and scr.
template <class Model>
__device__ __forceinline__ void point_phase(const ElemArgs& g, const double* s_g, const double* s_jxw, int64_t e, int q,
                                            bool live, double* P9, double* scr) {
  const int lane = threadIdx.x & 31;
  double uo[3] = {0.0, 0.0, 0.0};
  if (live) {
    const int64_t node = g.conn[e * 8 + q];
#pragma unroll
    for (int d = 0; d < 3; ++d) uo[d] = __ldg(&g.U[node * 3 + d]);
  }
  double gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  const double* gq = s_g + q * 24;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int src = (lane & ~7) | a;
    const double u0 = __shfl_sync(0xffffffffu, uo[0], src), u1 = __shfl_sync(0xffffffffu, uo[1], src),
                 u2 = __shfl_sync(0xffffffffu, uo[2], src);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double gj = gq[a * 3 + j];
      gu[0][j] = fma(u0, gj, gu[0][j]);
      gu[1][j] = fma(u1, gj, gu[1][j]);
      gu[2][j] = fma(u2, gj, gu[2][j]);
    }
  }
  if (live) {
    const double* so = Model::NS ? g.state_old + (e * NQ + q) * Model::NS : nullptr;
    double* sn = (Model::NS && g.state_new) ? g.state_new + (e * NQ + q) * Model::NS : nullptr;
    Model::point(g.props, gu, s_jxw[q], so, sn, P9, scr);
  }
}

// node pair n = (a, b), a <= b, as a << 4 | b
__constant__ unsigned char kPairNodes[NPAIR] = {0x00, 0x01, 0x02, 0x03, 0x04, 0x05, 0x06, 0x07, 0x11, 0x12, 0x13, 0x14, 0x15, 0x16, 0x17, 0x22, 0x23, 0x24, 0x25, 0x26, 0x27, 0x33, 0x34, 0x35, 0x36, 0x37, 0x44, 0x45, 0x46, 0x47, 0x55, 0x56, 0x57, 0x66, 0x67, 0x77};

// sum_L v_L[j] 2^(-8L) of the seven level accumulators of one pair: levels 6..4
// in FP32 (their rounding is below 2^-55 of level 0), then 3..0 in double-float
__device__ __forceinline__ float2 combine_levels(const float (&v)[NLEV][4], int j) {
  float hi = fmaf(fmaf(v[6][j], 0.00390625f, v[5][j]), 0.00390625f, v[4][j]), lo = 0.f;
#pragma unroll
  for (int L = 3; L >= 0; --L) {
    const float a = v[L][j], b = hi * 0.00390625f;
    lo *= 0.00390625f;
    const float s = a + b, bb = s - a;
    lo += (a - (s - bb)) + (b - bb);
    hi = s + lo;
    lo = lo - (hi - s);
  }
  return make_float2(hi, lo);
}

// R_(a,i) of one element from its points' split JxW P [8][9] (double-float, q in order)
__device__ __forceinline__ double residual_entry(const float2* s_g2, const float2* P8, int a, int i) {
  float2 R = make_float2(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const float2* gq = s_g2 + q * 24 + a * 3;
    const float2* P = P8 + q * 9 + i * 3;
    R = df64_dot3_acc(R, gq[0], P[0], gq[1], P[1], gq[2], P[2]);
  }
  return widen(R.x) + widen(R.y);
}

template <class Model, bool WANT_R>
__global__ void __launch_bounds__(NTHR, 1) hex8_affine_tc_kernel(ElemArgs g, const unsigned char* __restrict__ tab) {
  using namespace tc;
  using Lay = Layout<Model>;
  constexpr int SCR2 = Model::SCR2;
  extern __shared__ __align__(1024) unsigned char sm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s0 = smem_u32(sm);
  double* s_g = reinterpret_cast<double*>(sm + Lay::G);
  float2* s_g2 = reinterpret_cast<float2*>(sm + Lay::G2);
  double* s_jxw = reinterpret_cast<double*>(sm + Lay::JXW);
  int* s_sig = reinterpret_cast<int*>(sm + Lay::SIG);
  int* s_tau = reinterpret_cast<int*>(sm + Lay::TAU);
  int* s_taust = reinterpret_cast<int*>(sm + Lay::TAUST);
  uint32_t* s_code = reinterpret_cast<uint32_t*>(sm + Lay::CODE);
  uint64_t* bar_sl = reinterpret_cast<uint64_t*>(sm + Lay::BAR);  // slices of a tile written
  uint64_t* bar_mma = bar_sl + 1;                                  // a tile's MMAs complete
  uint64_t* bar_tfree = bar_sl + 2;                                // the epilogue read a tile's accumulators
  float2* s_P = reinterpret_cast<float2*>(sm + Lay::P);
  float2* s_scr = reinterpret_cast<float2*>(sm + Lay::SCR);

  // ---- setup: A slices zero (padding rows and columns stay zero), W digits, tables ----
  for (int i = tid; i < ND * A_SLICE / 16; i += NTHR)
    reinterpret_cast<uint4*>(sm + Lay::A)[i] = make_uint4(0u, 0u, 0u, 0u);
  for (int i = tid; i < ND * W_SLICE / 16; i += NTHR)
    reinterpret_cast<uint4*>(sm + Lay::W)[i] = __ldg(reinterpret_cast<const uint4*>(tab + T_W) + i);
  for (int i = tid; i < NQ * 24; i += NTHR) {
    const double v = __ldg(reinterpret_cast<const double*>(tab + T_G) + i);
    s_g[i] = v;
    s_g2[i] = df64_split(v);
  }
  if (tid < NQ) s_jxw[tid] = __ldg(reinterpret_cast<const double*>(tab + T_JXW) + tid);
  if (tid < NPAD) s_sig[tid] = __ldg(reinterpret_cast<const int*>(tab + T_SIG) + tid);
  if (tid < 45) {
    // unique entry w = (r1, r2), r1 <= r2, r1 = 3i + J, r2 = 3k + L: i, J, k, L and
    // the operand positions (row ik = 3i + k, column 3J + L) and (row 3k + i, column 3L + J)
    int m = tid, r = 0;
    for (int c = 0; c < 9; ++c)
      if (m >= 9 - r) { m -= 9 - r; ++r; }
    const int r1 = r, r2 = r + m;
    const int i = r1 / 3, J = r1 % 3, k = r2 / 3, L = r2 % 3;
    s_code[tid] = uint32_t(i) | uint32_t(J) << 4 | uint32_t(k) << 8 | uint32_t(L) << 12 |
                  uint32_t(i * 3 + k) << 16 | uint32_t(J * 3 + L) << 20 | uint32_t(k * 3 + i) << 24 |
                  uint32_t(L * 3 + J) << 28;
  }
  if (tid == 0) {
    mbar_init(bar_sl, NSL);
    mbar_init(bar_mma, 1);
    mbar_init(bar_tfree, 32 * EP_W);
    mbar_fence_init();
  }
  if (warp == T_EP / 32) tmem_alloc(reinterpret_cast<uint32_t*>(sm + Lay::TSLOT), TMEM_COLS);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + Lay::TSLOT);
  const int64_t ntiles = (g.ne + EPT - 1) / EPT;
  const long long budget = g.wait_budget > 0 ? g.wait_budget : WAIT_BUDGET;
  // a wait that gave up reports through the flag and waits again (the long
  // budget) so that no buffer is reused under an operation in flight
  auto wait_or_report = [&](uint64_t* bar, uint32_t par) {
    if (!mbar_wait(bar, par, budget)) {
      if (g.wait_err) atomicExch(g.wait_err, 1);
      mbar_wait(bar, par, WAIT_BUDGET);
    }
  };

  if (tid < T_SL) {
    // ---------------- producers: thread (el, q) ----------------
    const int el = tid >> 3, q = tid & 7;
    for (int k = 0;; ++k) {
      const int64_t tile = blockIdx.x + int64_t(k) * gridDim.x;
      if (tile >= ntiles) break;
      const int64_t e = tile * EPT + el;
      const bool live = e < g.ne;
      double P9[9], scr[Model::SCR];
      point_phase<Model>(g, s_g, s_jxw, e, q, live, P9, scr);
      if (k >= 1) named_sync(BAR_EMPTY, N_FULL);  // tile k-1's staging has been read
      float bnd = 0.f;
      if (live) {
        float2* pP = s_P + tid * 9;
#pragma unroll
        for (int m = 0; m < 9; ++m) pP[m] = df64_split(P9[m]);
        Model::split_scratch(scr, s_scr + tid * SCR2);
        bnd = Model::abound(s_scr + tid * SCR2) * 1.0001f;
      }
      // the element's scale 2^tau > |every tangent entry| (its eight points are
      // lanes 8j .. 8j+7 of this warp)
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) bnd = fmaxf(bnd, __shfl_xor_sync(0xffffffffu, bnd, o));
      if (q == 0) {
        int tau = 0;
        if (bnd > 0.f) frexpf(bnd, &tau);
        s_taust[el] = tau < -119 ? -119 : (tau > 126 ? 126 : tau);
      }
      named_arrive(BAR_FULL, N_FULL);
    }
  } else if (tid < T_R) {
    // ---------------- slicers: thread (point p, half h) ----------------
    const int ts = tid - T_SL, p = ts >> 1, h = ts & 1, el = p >> 3, q = p & 7;
    const int w0 = h ? 23 : 0, cnt = h ? 22 : 23;
    const int rbase = row_of(el, 0);
    // this warp's TMEM lanes (quarter warp % 4) and entry columns (two slicer warps share quarters 0 and 3)
    const uint32_t ent = tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t(TM_ENT + (warp >= 7 ? 48 : 0));
    for (int k = 0;; ++k) {
      const int64_t tile = blockIdx.x + int64_t(k) * gridDim.x;
      if (tile >= ntiles) break;
      const bool live = tile * EPT + el < g.ne;
      named_sync(BAR_FULL, N_FULL);
      const float2* sc = s_scr + p * SCR2;
      const int tau = s_taust[el];
      const float fs = pow2f(7 - tau);  // entries scaled to |x| < 128
      // pass 1 (overlaps the previous tile's MMAs): the scaled entries into this
      // lane's TMEM columns ent + 2c (hi), + 2c + 1 (lo); 23 steps on every lane
      // (the .sync.aligned stores), the 23rd a zero on the half with 22
#pragma unroll 1
      for (int c = 0; c < 23; c += 2) {
        const int c1 = c + 1 < 23 ? c + 1 : c;
        const uint32_t code0 = s_code[w0 + (c < cnt ? c : 0)], code1 = s_code[w0 + (c1 < cnt ? c1 : 0)];
        float2 a0 = make_float2(0.f, 0.f), a1 = a0;
        if (live && c < cnt)
          a0 = Model::aentry_df64(sc, code0 & 15, (code0 >> 4) & 15, (code0 >> 8) & 15, (code0 >> 12) & 15);
        if (live && c1 < cnt)
          a1 = Model::aentry_df64(sc, code1 & 15, (code1 >> 4) & 15, (code1 >> 8) & 15, (code1 >> 12) & 15);
        tmem_st2(ent + uint32_t(2 * c), a0.x * fs, a0.y * fs);
        if (c + 1 < 23) tmem_st2(ent + uint32_t(2 * c + 2), a1.x * fs, a1.y * fs);
      }
      tmem_wait_st();
      named_arrive(BAR_EMPTY, N_FULL);  // the staging may be refilled
      // pass 2: the digits, once tile k-1's MMAs have read the slices
      if (k >= 1) wait_or_report(bar_mma, uint32_t((k - 1) & 1));
      if ((ts & 15) == 0) s_tau[(k & 1) * 16 + el] = tau;
      unsigned char* As = sm + Lay::A;
#pragma unroll 1
      for (int c0 = 0; c0 < 24; c0 += 4) {
        float x[8];
        tmem_ld8(ent + uint32_t(2 * c0), x);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = c0 + j;
          if (c >= cnt) break;
          const uint32_t code = s_code[w0 + c];
          unsigned char* p1 = As + op_off(rbase + int((code >> 16) & 15), q * 9 + int((code >> 20) & 15));
          unsigned char* p2 = As + op_off(rbase + int((code >> 24) & 15), q * 9 + int(code >> 28));
          const bool twin = p1 != p2;
          float xh = x[2 * j], xl = x[2 * j + 1];
#pragma unroll
          for (int s = 0; s < ND; ++s) {
            const float dh = rintf(xh), dl = rintf(xl);
            xh = (xh - dh) * 256.f;
            xl = (xl - dl) * 256.f;
            const unsigned short bits = static_cast<unsigned short>(__float_as_uint(dh + dl) >> 16);
            *reinterpret_cast<unsigned short*>(p1 + s * A_SLICE) = bits;
            if (twin) *reinterpret_cast<unsigned short*>(p2 + s * A_SLICE) = bits;
          }
        }
      }
      fence_async_smem();
      mbar_arrive(bar_sl);
    }
  } else if (tid < T_EP) {
    // ---------------- residual warp ----------------
    for (int k = 0;; ++k) {
      const int64_t tile = blockIdx.x + int64_t(k) * gridDim.x;
      if (tile >= ntiles) break;
      named_sync(BAR_FULL, N_FULL);
      if (WANT_R) {
        static_assert(EPT * 24 % 32 == 0, "residual entries per lane");
#pragma unroll 3
        for (int j = 0; j < EPT * 24 / 32; ++j) {
          const int idx = lane + 32 * j, el = idx / 24, ai = idx % 24;
          const int64_t e = tile * EPT + el;
          const double r = residual_entry(s_g2, s_P + el * NQ * 9, ai / 3, ai % 3);
          if (e < g.ne) static_cast<double*>(g.Re)[e * 24 + ai] = r;
        }
      }
      named_arrive(BAR_EMPTY, N_FULL);
    }
  } else if (tid < T_MMA) {
    // ---------------- epilogue: thread = TMEM lane = row (el, i, k) ----------------
    const int qw = warp & 3;
    const int el = qw * 3 + (lane < 27 ? lane / 9 : 0), ik = lane % 9, i = ik / 3, kc = ik % 3;
    const uint32_t lane_addr = tmem + (uint32_t(qw * 32) << 16);
    for (int k = 0;; ++k) {
      const int64_t tile = blockIdx.x + int64_t(k) * gridDim.x;
      if (tile >= ntiles) break;
      const uint32_t par = uint32_t(k & 1);
      wait_or_report(bar_sl, par);
      wait_or_report(bar_mma, par);
      tc_fence_after();
      const int64_t e0 = tile * EPT;
      const bool live = lane < 27 && e0 + el < g.ne;
      const int tau = s_tau[(k & 1) * 16 + el];
      const float f1 = pow2f(tau - 7);
      if (g.ke_pairs) {
        // the symmetric half straight from the levels: pair n = (a, b) of row
        // (el, i, k) is K_(a,i),(b,k), entry 9n + 3i + k of the element's KE_PAIRS block
        float2* dst = static_cast<float2*>(g.Ke) + (e0 + el) * (NPAIR * 9) + ik;
#pragma unroll 1
        for (int c = 0; c < NPAIR / 4; ++c) {
          float v[NLEV][4];
          tmem_ld4x7(lane_addr + uint32_t(c * 4), v);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float2 hl = combine_levels(v, j);
            const float f = f1 * pow2f(s_sig[c * 4 + j] - 7);
            if (live) dst[(c * 4 + j) * 9] = make_float2(hl.x * f, hl.y * f);
          }
        }
        tc_fence_before();
        mbar_arrive(bar_tfree);  // the accumulators may be overwritten
        continue;
      }
      // node rows of the whole K_e: pair n = (a, b) of row (el, i, k), K_(a,i),(b,k), is
      // entry b of node row (a, i, k) and, by symmetry, entry a of node row (b, k, i)
      float2* dst = static_cast<float2*>(g.Ke) + (e0 + el) * 576;
#pragma unroll 1
      for (int c = 0; c < NPAIR / 4; ++c) {
        float v[NLEV][4];
        tmem_ld4x7(lane_addr + uint32_t(c * 4), v);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float2 hl = combine_levels(v, j);
          const float f = f1 * pow2f(s_sig[c * 4 + j] - 7);
          const int ab = kPairNodes[c * 4 + j], a = ab >> 4, b = ab & 15;
          const float2 val = make_float2(hl.x * f, hl.y * f);
          if (live) {
            dst[((a * 3 + i) * 3 + kc) * 8 + b] = val;
            if (a != b) dst[((b * 3 + kc) * 3 + i) * 8 + a] = val;
          }
        }
      }
      tc_fence_before();
      mbar_arrive(bar_tfree);  // the accumulators may be overwritten
    }
  } else {
    // ---------------- MMA warp: lane 0 issues, the warp waits together ----------------
    const uint32_t aB = s0 + Lay::A, wB = s0 + Lay::W;
    const uint64_t dA = smem_desc(aB, 128, SBO), dW = smem_desc(wB, 128, SBO);
    for (int k = 0;; ++k) {
      const int64_t tile = blockIdx.x + int64_t(k) * gridDim.x;
      if (tile >= ntiles) break;
      if (k >= 1) wait_or_report(bar_tfree, uint32_t((k - 1) & 1));  // the accumulators are free
      wait_or_report(bar_sl, uint32_t(k & 1));                       // the tile's slices are written
      tc_fence_after();
      if (lane == 0) {
#pragma unroll 1
        for (int gi = 0; gi < NGROUP; ++gi) {
          const int t = kGroups[gi][0], s0g = kGroups[gi][1], ns = kGroups[gi][2];
          const uint32_t idesc = tc::idesc_bf16(128, NPAD * ns), d = tmem + uint32_t((s0g + t) * NPAD);
          const uint64_t a0 = dA + uint64_t((t * A_SLICE) >> 4), w0d = dW + uint64_t((s0g * W_SLICE) >> 4);
#pragma unroll
          for (int kk = 0; kk < KP / 16; ++kk)
            mma_bf16(d, a0 + uint64_t(kk * 16), w0d + uint64_t(kk * 16), idesc, (t == 0 && kk == 0) ? 0u : 1u);
        }
        mma_commit(bar_mma);
      }
      __syncwarp();
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == T_EP / 32) {
    tc_fence_after();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// Residual only (no tangent): the same point phase and residual arithmetic as
// the tensor-core kernel, so both give bitwise the same R and state.  16
// elements per CTA, one thread per point.
constexpr int R_EPB = 16;
template <class Model>
__global__ void __launch_bounds__(R_EPB * NQ) hex8_affine_r_kernel(ElemArgs g, const unsigned char* __restrict__ tab) {
  __shared__ double s_g[NQ * 24], s_jxw[NQ];
  __shared__ float2 s_g2[NQ * 24], s_P[R_EPB * NQ * 9];
  const int tid = threadIdx.x, el = tid >> 3, q = tid & 7;
  for (int i = tid; i < NQ * 24; i += blockDim.x) {
    const double v = __ldg(reinterpret_cast<const double*>(tab + T_G) + i);
    s_g[i] = v;
    s_g2[i] = df64_split(v);
  }
  if (tid < NQ) s_jxw[tid] = __ldg(reinterpret_cast<const double*>(tab + T_JXW) + tid);
  __syncthreads();
  const int64_t e0 = int64_t(blockIdx.x) * R_EPB, e = e0 + el;
  const bool live = e < g.ne;
  double P9[9], scr[Model::SCR];
  point_phase<Model>(g, s_g, s_jxw, e, q, live, P9, scr);
  if (live) {
#pragma unroll
    for (int m = 0; m < 9; ++m) s_P[tid * 9 + m] = df64_split(P9[m]);
  }
  __syncthreads();
  for (int idx = tid; idx < R_EPB * 24; idx += blockDim.x) {
    const int ee = idx / 24, ai = idx % 24;
    if (e0 + ee < g.ne)
      static_cast<double*>(g.Re)[(e0 + ee) * 24 + ai] = residual_entry(s_g2, s_P + ee * NQ * 9, ai / 3, ai % 3);
  }
}

template <class Model, bool WANT_R>
cudaError_t launch1(const ElemArgs& a, cudaStream_t s, int* launches) {
  constexpr int SMEM = Layout<Model>::SMEM;
  const cudaError_t e = ensure_smem<hex8_affine_tc_kernel<Model, WANT_R>>(SMEM);
  if (e != cudaSuccess) return e;
  const int64_t ntiles = (a.ne + EPT - 1) / EPT;
  if (ntiles == 0) return cudaSuccess;
  const int grid = int(ntiles < num_sms() ? ntiles : num_sms());
  hex8_affine_tc_kernel<Model, WANT_R><<<grid, NTHR, SMEM, s>>>(a, static_cast<const unsigned char*>(a.affine));
  if (launches) ++*launches;
  return cudaGetLastError();
}

template <class Model>
cudaError_t launch_r(const ElemArgs& a, cudaStream_t s, int* launches) {
  const int64_t nb = (a.ne + R_EPB - 1) / R_EPB;
  if (nb == 0) return cudaSuccess;
  hex8_affine_r_kernel<Model><<<unsigned(nb), R_EPB * NQ, 0, s>>>(a, static_cast<const unsigned char*>(a.affine));
  if (launches) ++*launches;
  return cudaGetLastError();
}

}  // namespace aff

bool hex8_affine_enabled() {
  const char* v = std::getenv("FEC_HEX8_AFFINE");
  return !(v && v[0] == '0');
}

size_t hex8_affine_grad_offset() {
  static_assert(aff::T_JXW == aff::T_G + aff::NQ * 24 * 8, "gradients, then JxW");
  return size_t(aff::T_G);
}

bool hex8_pairs_enabled() {
  const char* v = std::getenv("FEC_HEX8_PAIRS");
  return !(v && v[0] == '0');
}

cudaError_t launch_hex8_affine_tc(int physics, bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s,
                                  int* launches) {
  if (!a.affine || (want_k && !a.Ke) || (want_r && !a.Re)) return cudaErrorInvalidValue;
  if (!want_k) {
    if (!want_r) return cudaSuccess;
    if (physics == 2) return aff::launch_r<NeoHookean>(a, s, launches);
    if (physics == 3) return aff::launch_r<J2>(a, s, launches);
    return cudaErrorNotSupported;
  }
  if (physics == 2)
    return want_r ? aff::launch1<NeoHookean, true>(a, s, launches) : aff::launch1<NeoHookean, false>(a, s, launches);
  if (physics == 3) return want_r ? aff::launch1<J2, true>(a, s, launches) : aff::launch1<J2, false>(a, s, launches);
  return cudaErrorNotSupported;
}

// Host: the constant operand of a block whose elements are translates of its
// first one.  x0: the first element's node coordinates [8][3]; ref: the block's
// reference tables (RefLayout<1>: N, dN/dxi [q][a][3], weights).  Returns false
// for a degenerate element (det J <= 0 at a point) or gradient products outside
// the range the FP32 epilogue scales (2^-126 .. 2^127).
bool hex8_affine_table(const double* x0, const double* ref, std::vector<unsigned char>& out) {
  using L = RefLayout<1>;
  out.assign(aff::T_BYTES, 0);
  double dNX[8][8][3], jxw[8];
  for (int q = 0; q < 8; ++q) {
    const double* dN = ref + L::DN_OFF + q * 24;
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d)
        for (int k = 0; k < 3; ++k) J[d][k] = std::fma(x0[a * 3 + d], dN[a * 3 + k], J[d][k]);
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2],
                 c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    if (!(det > 0.0)) return false;
    const double r = 1.0 / det;
    double Ji[3][3];
    Ji[0][0] = c00 * r;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
    Ji[1][0] = c01 * r;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
    Ji[2][0] = c02 * r;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s = std::fma(dN[a * 3 + k], Ji[k][d], s);
        dNX[q][a][d] = s;
      }
    jxw[q] = det * ref[L::W_OFF + q];
  }
  int n = 0;
  int32_t sig[aff::NPAD] = {0};
  for (int a = 0; a < 8; ++a)
    for (int b = a; b < 8; ++b, ++n) {
      double w[aff::KR], mx = 0.0;
      for (int q = 0; q < 8; ++q)
        for (int J = 0; J < 3; ++J)
          for (int Lc = 0; Lc < 3; ++Lc) {
            w[q * 9 + J * 3 + Lc] = dNX[q][a][J] * dNX[q][b][Lc];
            mx = std::fmax(mx, std::fabs(w[q * 9 + J * 3 + Lc]));
          }
      int e = 0;
      if (mx > 0.0) std::frexp(mx, &e);  // |w| < 2^e
      if (e < -119 || e > 134) return false;  // the epilogue scales by 2^(e - 7) in FP32
      sig[n] = e;
      for (int r = 0; r < aff::KR; ++r) {
        double y = std::ldexp(w[r], 7 - e);  // |y| < 128, exact
        for (int s = 0; s < aff::ND; ++s) {
          const double d = std::nearbyint(y);
          y = (y - d) * 256.0;
          const float fd = float(d);
          uint32_t u;
          std::memcpy(&u, &fd, 4);
          const uint16_t bits = uint16_t(u >> 16);
          std::memcpy(out.data() + aff::T_W + s * aff::W_SLICE + aff::op_off(n, r), &bits, 2);
        }
      }
    }
  std::memcpy(out.data() + aff::T_SIG, sig, sizeof sig);
  std::memcpy(out.data() + aff::T_G, dNX, sizeof dNX);
  std::memcpy(out.data() + aff::T_JXW, jxw, sizeof jxw);
  return true;
}

}  // namespace fec
