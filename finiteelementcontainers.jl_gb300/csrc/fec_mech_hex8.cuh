// fec_mech_hex8.cuh -- the hex8 mechanics element kernel used for the
// benchmark workloads (vector hex8, 2x2x2 points, symmetric tangent).
//
// Compared with the generic mech_element_kernel (one thread per element row):
//  * the tangent is symmetric for the hyperelastic and associative-plastic
//    models here (A_iJkL = A_kLiJ), so only 36 of the 64 node-pair blocks of
//    K_e are contracted (32% fewer FMAs): in the FP32/FP64 kernels each
//    element is served by 12 threads, thread (p, i) owning rows (p, i) and
//    (7-p, i) and the column blocks b >= row node (9 blocks per thread); the
//    df64 kernel uses 24 threads per element with a circulant cover (below);
//  * the tangent tensor is evaluated from its 45 unique entries;
//  * K_e is staged in shared memory (the mirrored half written there) in the
//    KE_NODE_ROWS layout the node gather reads, and leaves the CTA as one
//    contiguous, 16-byte vectorised stream;
//  * in the FP32-element variant the isoparametric map runs in FP32 on
//    coordinate differences taken in FP64 (x_a - x_0), with the FP64 map kept
//    for distorted elements (Hadamard ratio |det J| / prod |J col| < 0.25), so
//    the FP64 pipe no longer carries the per-point kinematics.
#pragma once
#include <type_traits>
#include "fec_kernels.cuh"
#include "fec_tc.cuh"

namespace fec {

// Stages the hex8 reference tables (shape-function values and gradients, 264
// doubles) and the connectivity of the CTA's `nlive` elements into shared
// memory with bulk (TMA) copies that complete on an mbarrier.  Connectivity of
// a block that does not start on a 16-byte boundary falls back to plain loads.
// A wait that gives up (after `budget` SM clocks, 0: about 1 s) sets *err,
// waits once more (about 1 s) so that no copy lands after the CTA has moved
// on, and then loads with plain loads.  Ends with a barrier.
__device__ __forceinline__ void stage_hex8_tables(const double* gref, double* s_ref, const int32_t* gconn, int nlive,
                                                  int* s_conn, uint64_t* bar, int tid, int nthr, int* err,
                                                  long long budget, bool allow_bulk = true) {
  constexpr int NREF = RefLayout<1>::SIZE;
  const bool bulk =
      allow_bulk && ((reinterpret_cast<uintptr_t>(gref) | reinterpret_cast<uintptr_t>(gconn)) & 15) == 0;
  bool done = false;
  if (bulk) {
    if (tid == 0) {
      tc::mbar_init(bar, 1);
      tc::mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0) {
      tc::mbar_expect_tx(bar, uint32_t(NREF * 8 + nlive * 32));
      tc::bulk_g2s(s_ref, gref, NREF * 8, bar);
      tc::bulk_g2s(s_conn, gconn, uint32_t(nlive * 32), bar);
    }
    const bool landed = tc::mbar_wait(bar, 0, budget > 0 ? budget : 2000000000LL);
    if (__syncthreads_or(!landed)) {
      if (tid == 0 && err) atomicExch(err, 1);
      tc::mbar_wait(bar, 0, 2000000000LL);
    } else {
      done = true;
    }
  }
  if (!done) {
    for (int i = tid; i < NREF; i += nthr) s_ref[i] = gref[i];
    for (int i = tid; i < nlive * 8; i += nthr) s_conn[i] = gconn[i];
  }
  __syncthreads();
}

// (r1, r2), r1 <= r2, of the m-th unique entry of a symmetric 9x9 matrix
__device__ __forceinline__ void sym_pair(int m, int& r1, int& r2) {
  int r = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int cnt = 9 - r;
    if (m >= cnt) {
      m -= cnt;
      ++r;
    }
  }
  r1 = r;
  r2 = r + m;
}

// Packed upper-triangle index of entry (r1, r2) of a symmetric 9x9 matrix (the
// order sym_pair enumerates).
__device__ __forceinline__ int sym_index(int r1, int r2) {
  const int lo = r1 < r2 ? r1 : r2, hi = r1 < r2 ? r2 : r1;
  return 9 * lo - (lo * (lo - 1)) / 2 + (hi - lo);
}

// FP32 map of a hex8 point from FP64-differenced coordinates; falls back to the
// FP64 map for distorted elements.  Returns JxW.
__device__ __forceinline__ float map_hex8_mixed(const double* __restrict__ s_ref, const float* __restrict__ s_reff,
                                                int q, const double* __restrict__ x, const float* __restrict__ xd,
                                                float* __restrict__ dNX) {
  using L = RefLayout<1>;
  const float* dN = s_reff + L::DN_OFF + q * 24;
  float J[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
  for (int a = 1; a < 8; ++a)  // xd[0] = 0
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int k = 0; k < 3; ++k) J[d][k] = fmaf(xd[a * 3 + d], dN[a * 3 + k], J[d][k]);
  const float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const float c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const float c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const float det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  float n0 = 0.f, n1 = 0.f, n2 = 0.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    n0 = fmaf(J[d][0], J[d][0], n0);
    n1 = fmaf(J[d][1], J[d][1], n1);
    n2 = fmaf(J[d][2], J[d][2], n2);
  }
  if (!(fabsf(det) >= 0.25f * sqrtf(n0 * n1 * n2))) return float(map_point<1, float>(s_ref, q, x, dNX, nullptr));
  const float r = 1.0f / det;
  float Ji[3][3];
  Ji[0][0] = c00 * r;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
  Ji[1][0] = c01 * r;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
  Ji[2][0] = c02 * r;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      dNX[a * 3 + d] = fmaf(dN[a * 3 + 0], Ji[0][d], fmaf(dN[a * 3 + 1], Ji[1][d], dN[a * 3 + 2] * Ji[2][d]));
  return det * float(s_ref[L::W_OFF + q]);
}

template <class Model, typename Real, int EPB>
struct Hex8Smem {
  static constexpr int NQ = 8, SCR = Model::SCR;
  static constexpr int REF = RefLayout<1>::SIZE;                   // 264
  static constexpr int D_REF = 0, D_X = D_REF + REF;                // doubles
  static constexpr int N_DOUBLE = D_X + EPB * 24;
  static constexpr int R_REFF = 0;                                  // Reals, after the doubles
  static constexpr int R_XD = R_REFF + REF;
  static constexpr int R_U = R_XD + EPB * 24;
  static constexpr int R_DNX = R_U + EPB * 24;
  // per-element stride of the spatial gradients, padded by 8 words: a warp spans
  // up to 3 elements reading the same offset, which then fall in distinct banks
  static constexpr int DNX_STRIDE = NQ * 24 + (sizeof(Real) == 4 ? 8 : 4);
  static constexpr int R_JXW = R_DNX + EPB * DNX_STRIDE;
  static constexpr int R_P = R_JXW + EPB * NQ;
  static constexpr int R_SCR = R_P + EPB * NQ * 9;
  static constexpr int R_A = (R_SCR + EPB * NQ * SCR + 3) & ~3;     // 16-byte aligned for the vector copy-out
  static constexpr int A_STRIDE = NQ * 81;                          // per element; >= 576 for the K staging
  static constexpr int N_REAL = R_A + EPB * A_STRIDE;
  static constexpr size_t BYTES = sizeof(double) * N_DOUBLE + sizeof(Real) * N_REAL + sizeof(int) * EPB * 8 + 16;
};

template <class Model, typename Real, int EPB, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(EPB * 12) mech_hex8_sym_kernel(ElemArgs g) {
  constexpr int NQ = 8, TPE = 12, NS = Model::NS, SCR = Model::SCR;
  constexpr bool F64 = std::is_same<Real, double>::value;
  using S = Hex8Smem<Model, Real, EPB>;
  using L = RefLayout<1>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s_ref = reinterpret_cast<double*>(smem_raw) + S::D_REF;
  double* s_x_all = reinterpret_cast<double*>(smem_raw) + S::D_X;
  Real* rb = reinterpret_cast<Real*>(reinterpret_cast<double*>(smem_raw) + S::N_DOUBLE);
  Real* s_reff = rb + S::R_REFF;
  int* s_conn_all = reinterpret_cast<int*>(rb + S::N_REAL);

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * TPE + tx, nthr = EPB * TPE;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int64_t e = e0 + ty;
  const bool live = e < g.ne;
  double* s_x = s_x_all + ty * 24;
  Real* s_xd = rb + S::R_XD + ty * 24;
  Real* s_u = rb + S::R_U + ty * 24;
  Real* s_dNX = rb + S::R_DNX + ty * S::DNX_STRIDE;
  Real* s_jxw = rb + S::R_JXW + ty * NQ;
  Real* s_P = rb + S::R_P + ty * NQ * 9;
  Real* s_scr = rb + S::R_SCR + ty * NQ * SCR;
  Real* s_A = rb + S::R_A + ty * S::A_STRIDE;
  int* s_conn = s_conn_all + ty * 8;

  for (int i = tid; i < L::SIZE; i += nthr) {
    const double v = g.ref[i];
    s_ref[i] = v;
    if (!F64) s_reff[i] = Real(v);
  }
  if (live && tx < 8) s_conn[tx] = g.conn[e * 8 + tx];
  __syncthreads();
  if (live) {
    for (int i = tx; i < 24; i += TPE) {
      const int a = i / 3, d = i % 3;
      const double xv = __ldg(&g.coords[int64_t(s_conn[a]) * 3 + d]);
      s_x[i] = xv;
      if (!F64) s_xd[i] = Real(xv - __ldg(&g.coords[int64_t(s_conn[0]) * 3 + d]));
      s_u[i] = Real(__ldg(&g.U[int64_t(s_conn[a]) * 3 + d]));
    }
  }
  __syncthreads();

  // per-point kinematics and constitutive update
  if (live && tx < NQ) {
    const int q = tx;
    Real* dNX = s_dNX + q * 24;
    Real jxw;
    if constexpr (F64)
      jxw = Real(map_point<1, double>(s_ref, q, s_x, dNX, nullptr));
    else
      jxw = map_hex8_mixed(s_ref, s_reff, q, s_x, s_xd, dNX);
    s_jxw[q] = jxw;
    Real gu[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        Real s = 0;
#pragma unroll
        for (int a = 0; a < 8; ++a) s = fma(s_u[a * 3 + i], dNX[a * 3 + j], s);
        gu[i][j] = s;
      }
    const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
    double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
    Model::point(g.props, gu, jxw, so, sn, s_P + q * 9, s_scr + q * SCR);
  }
  __syncthreads();
  // JxW-scaled tangent from its 45 unique entries
  if (WANT_K && live) {
    for (int w = tx; w < NQ * 45; w += TPE) {
      const int q = w / 45;
      int r1, r2;
      sym_pair(w - q * 45, r1, r2);
      const Real v = Model::aentry(s_scr + q * SCR, r1 / 3, r1 % 3, r2 / 3, r2 % 3);
      Real* Aq = s_A + q * 81;
      Aq[r1 * 9 + r2] = v;
      Aq[r2 * 9 + r1] = v;
    }
  }
  __syncthreads();

  const int pp = tx / 3, i = tx % 3;
  const int a1 = pp, a2 = 7 - pp;
  const int split = 8 - pp;  // blocks j < split belong to row node a1
  Real K[27];
#pragma unroll
  for (int c = 0; c < 27; ++c) K[c] = 0;
  Real R1 = 0, R2 = 0;
  if (live) {
    for (int q = 0; q < NQ; ++q) {
      const Real* dNX = s_dNX + q * 24;
      const Real g10 = dNX[a1 * 3], g11 = dNX[a1 * 3 + 1], g12 = dNX[a1 * 3 + 2];
      const Real g20 = dNX[a2 * 3], g21 = dNX[a2 * 3 + 1], g22 = dNX[a2 * 3 + 2];
      if (WANT_R) {
        const Real* P = s_P + q * 9 + i * 3;
        R1 = fma(g10, P[0], fma(g11, P[1], fma(g12, P[2], R1)));
        R2 = fma(g20, P[0], fma(g21, P[1], fma(g22, P[2], R2)));
      }
      if (WANT_K) {
        const Real* Ai = s_A + q * 81 + i * 27;
        Real t1[9], t2[9];
#pragma unroll
        for (int kl = 0; kl < 9; ++kl) {
          const Real x0 = Ai[kl], x1 = Ai[9 + kl], x2 = Ai[18 + kl];
          t1[kl] = fma(g10, x0, fma(g11, x1, g12 * x2));
          t2[kl] = fma(g20, x0, fma(g21, x1, g22 * x2));
        }
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const bool first = j < split;
          const int b = first ? pp + j : j - 1;
          const Real h0 = dNX[b * 3], h1 = dNX[b * 3 + 1], h2 = dNX[b * 3 + 2];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const Real u0 = first ? t1[k * 3] : t2[k * 3];
            const Real u1 = first ? t1[k * 3 + 1] : t2[k * 3 + 1];
            const Real u2 = first ? t1[k * 3 + 2] : t2[k * 3 + 2];
            K[j * 3 + k] += fma(u0, h0, fma(u1, h1, u2 * h2));
          }
        }
      }
    }
  }
  __syncthreads();  // s_A is reused for the K staging below
  if (WANT_K && live) {
    using W = typename WS<Real>::T;
    W* Ks = reinterpret_cast<W*>(s_A);  // 576 entries, KE_NODE_ROWS layout ((a*3 + k)*3 + i)*8 + b
#pragma unroll
    for (int j = 0; j < 9; ++j) {
      const bool first = j < split;
      const int an = first ? a1 : a2;
      const int b = first ? pp + j : j - 1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const W w = WS<Real>::from(K[j * 3 + k]);
        Ks[((an * 3 + i) * 3 + k) * 8 + b] = w;
        if (b != an) Ks[((b * 3 + k) * 3 + i) * 8 + an] = w;
      }
    }
  }
  if (WANT_R && live) {
    Real* Re = static_cast<Real*>(g.Re) + e * 24;
    Re[a1 * 3 + i] = R1;
    Re[a2 * 3 + i] = R2;
  }
  if (WANT_K) {
    __syncthreads();
    using V = typename std::conditional<sizeof(Real) == 4, float4, double2>::type;
    constexpr int VW = 16 / sizeof(Real);
    constexpr int PER = 576 / VW;
    const int64_t left = g.ne - e0;
    const int nlive = left < EPB ? int(left) : EPB;
    V* dst = reinterpret_cast<V*>(static_cast<Real*>(g.Ke) + e0 * 576);
    const Real* src = rb + S::R_A;
    for (int idx = tid; idx < nlive * PER; idx += nthr) {
      const int el = idx / PER, off = idx - el * PER;
      dst[idx] = *reinterpret_cast<const V*>(src + el * S::A_STRIDE + off * VW);
    }
  }
}

// ---------------------------------------------------------------------------
// FP32-element variant.  On the FP32 pipes the contraction FMAs are cheap and
// integer/select work is what limits the symmetric kernel, so here each of the
// 12 threads of an element owns two full rows (p, i) and (p+4, i) over all 8
// column blocks: 57 shared-memory loads per 198 FMAs per point, every index a
// compile-time constant, no selects.  The tangent slice A_i... of a point is
// produced by one thread with i fixed at compile time.
// ---------------------------------------------------------------------------
template <class Model, typename Real, int I>
__device__ __forceinline__ void tangent_slice(const Real* scr, Real* out) {
#pragma unroll
  for (int J = 0; J < 3; ++J)
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int L = 0; L < 3; ++L) out[J * 9 + k * 3 + L] = Model::aentry(scr, I, J, k, L);
}

template <class Model, int EPB, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(EPB * 12) mech_hex8_rows2_kernel(ElemArgs g) {
  using Real = float;
  constexpr int NQ = 8, TPE = 12, NS = Model::NS, SCR = Model::SCR;
  using S = Hex8Smem<Model, Real, EPB>;
  using L = RefLayout<1>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* s_ref = reinterpret_cast<double*>(smem_raw) + S::D_REF;
  double* s_x_all = reinterpret_cast<double*>(smem_raw) + S::D_X;
  Real* rb = reinterpret_cast<Real*>(reinterpret_cast<double*>(smem_raw) + S::N_DOUBLE);
  Real* s_reff = rb + S::R_REFF;
  int* s_conn_all = reinterpret_cast<int*>(rb + S::N_REAL);

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * TPE + tx, nthr = EPB * TPE;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int64_t e = e0 + ty;
  const bool live = e < g.ne;
  double* s_x = s_x_all + ty * 24;
  Real* s_xd = rb + S::R_XD + ty * 24;
  Real* s_u = rb + S::R_U + ty * 24;
  Real* s_dNX = rb + S::R_DNX + ty * S::DNX_STRIDE;
  Real* s_P = rb + S::R_P + ty * NQ * 9;
  Real* s_scr = rb + S::R_SCR + ty * NQ * SCR;
  Real* s_A = rb + S::R_A + ty * S::A_STRIDE;
  int* s_conn = s_conn_all + ty * 8;

  {
    const int64_t left = g.ne - e0;
    stage_hex8_tables(g.ref, s_ref, g.conn + e0 * 8, left < EPB ? int(left) : EPB, s_conn_all,
                      reinterpret_cast<uint64_t*>(s_conn_all + EPB * 8), tid, nthr, g.wait_err, g.wait_budget);
  }
  for (int i = tid; i < L::SIZE; i += nthr) s_reff[i] = Real(s_ref[i]);
  if (live) {
    for (int i = tx; i < 24; i += TPE) {
      const int a = i / 3, d = i % 3;
      const double xv = __ldg(&g.coords[int64_t(s_conn[a]) * 3 + d]);
      s_x[i] = xv;
      s_xd[i] = Real(xv - __ldg(&g.coords[int64_t(s_conn[0]) * 3 + d]));
      s_u[i] = Real(__ldg(&g.U[int64_t(s_conn[a]) * 3 + d]));
    }
  }
  __syncthreads();
  if (live && tx < NQ) {
    const int q = tx;
    Real* dNX = s_dNX + q * 24;
    const Real jxw = map_hex8_mixed(s_ref, s_reff, q, s_x, s_xd, dNX);
    Real gu[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        Real s = 0;
#pragma unroll
        for (int a = 0; a < 8; ++a) s = fmaf(s_u[a * 3 + i], dNX[a * 3 + j], s);
        gu[i][j] = s;
      }
    if constexpr (Model::USES_TABLE) {
      // constitutive response precomputed per point (by the closure kernel)
      Model::point_table(g.closure, e * NQ + q, jxw, s_P + q * 9, s_scr + q * SCR);
    } else {
      const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
      double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
      Model::point(g.props, gu, jxw, so, sn, s_P + q * 9, s_scr + q * SCR);
    }
  }
  __syncthreads();
  const int pp = tx / 3, i = tx % 3;
  if (WANT_K && live) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int q = pp + 4 * h;
      const Real* scr = s_scr + q * SCR;
      Real* out = s_A + q * 81 + i * 27;
      if (i == 0) tangent_slice<Model, Real, 0>(scr, out);
      else if (i == 1) tangent_slice<Model, Real, 1>(scr, out);
      else tangent_slice<Model, Real, 2>(scr, out);
    }
  }
  __syncthreads();
  const int a1 = pp, a2 = pp + 4;
  Real K1[24], K2[24];
#pragma unroll
  for (int c = 0; c < 24; ++c) K1[c] = K2[c] = 0.f;
  Real R1 = 0.f, R2 = 0.f;
  if (live) {
    for (int q = 0; q < NQ; ++q) {
      const Real* dNX = s_dNX + q * 24;
      const Real g10 = dNX[a1 * 3], g11 = dNX[a1 * 3 + 1], g12 = dNX[a1 * 3 + 2];
      const Real g20 = dNX[a2 * 3], g21 = dNX[a2 * 3 + 1], g22 = dNX[a2 * 3 + 2];
      if (WANT_R) {
        const Real* P = s_P + q * 9 + i * 3;
        R1 = fmaf(g10, P[0], fmaf(g11, P[1], fmaf(g12, P[2], R1)));
        R2 = fmaf(g20, P[0], fmaf(g21, P[1], fmaf(g22, P[2], R2)));
      }
      if (WANT_K) {
        const Real* Ai = s_A + q * 81 + i * 27;
        Real t1[9], t2[9];
#pragma unroll
        for (int kl = 0; kl < 9; ++kl) {
          const Real x0 = Ai[kl], x1 = Ai[9 + kl], x2 = Ai[18 + kl];
          t1[kl] = fmaf(g10, x0, fmaf(g11, x1, g12 * x2));
          t2[kl] = fmaf(g20, x0, fmaf(g21, x1, g22 * x2));
        }
#pragma unroll
        for (int b = 0; b < 8; ++b) {
          const Real h0 = dNX[b * 3], h1 = dNX[b * 3 + 1], h2 = dNX[b * 3 + 2];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            K1[b * 3 + k] += fmaf(t1[k * 3], h0, fmaf(t1[k * 3 + 1], h1, t1[k * 3 + 2] * h2));
            K2[b * 3 + k] += fmaf(t2[k * 3], h0, fmaf(t2[k * 3 + 1], h1, t2[k * 3 + 2] * h2));
          }
        }
      }
    }
  }
  __syncthreads();  // s_A is reused for the K staging below
  if (WANT_K && live) {
    // KE_NODE_ROWS layout: ((a*3 + k)*3 + i)*8 + b, column node b fastest
    float4* r1 = reinterpret_cast<float4*>(s_A + (a1 * 3 + i) * 24);
    float4* r2 = reinterpret_cast<float4*>(s_A + (a2 * 3 + i) * 24);
#pragma unroll
    for (int kc = 0; kc < 3; ++kc) {
      r1[2 * kc] = make_float4(K1[kc], K1[3 + kc], K1[6 + kc], K1[9 + kc]);
      r1[2 * kc + 1] = make_float4(K1[12 + kc], K1[15 + kc], K1[18 + kc], K1[21 + kc]);
      r2[2 * kc] = make_float4(K2[kc], K2[3 + kc], K2[6 + kc], K2[9 + kc]);
      r2[2 * kc + 1] = make_float4(K2[12 + kc], K2[15 + kc], K2[18 + kc], K2[21 + kc]);
    }
  }
  if (WANT_R && live) {
    Real* Re = static_cast<Real*>(g.Re) + e * 24;
    Re[a1 * 3 + i] = R1;
    Re[a2 * 3 + i] = R2;
  }
  if (WANT_K) {
    __syncthreads();
    constexpr int PER = 576 / 4;
    const int64_t left = g.ne - e0;
    const int nlive = left < EPB ? int(left) : EPB;
    float4* dst = reinterpret_cast<float4*>(static_cast<Real*>(g.Ke) + e0 * 576);
    const Real* src = rb + S::R_A;
    for (int idx = tid; idx < nlive * PER; idx += nthr) {
      const int el = idx / PER, off = idx - el * PER;
      dst[idx] = *reinterpret_cast<const float4*>(src + el * S::A_STRIDE + off * 4);
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 variant with the contraction on the FP32 pipes.  Kinematics and the
// constitutive update stay in FP64; the shape-function gradients, the stress and
// the tangent scratch are split into double-float (hi + lo) once per point, the
// tangent entries and the whole K_e / R_e contraction run in df64, and the
// double-float results go to the workspace as they are.
// ---------------------------------------------------------------------------
template <class Model, int EPB>
struct Hex8Df64Smem {
  static constexpr int NQ = 8, SCR2 = Model::SCR2;
  static constexpr int REF = RefLayout<1>::SIZE;
  static constexpr int D_REF = 0, D_X = REF, D_U = D_X + EPB * 24;
  static constexpr int N_DOUBLE = D_U + EPB * 24;
  static constexpr int F_DNX = 0;                       // float2 entries, after the doubles
  static constexpr int DNXS = NQ * 24 + 4;              // per element, padded (distinct banks across elements)
  static constexpr int F_P = F_DNX + EPB * DNXS;
  static constexpr int F_SCR = F_P + EPB * NQ * 9;
  static constexpr int F_A = (F_SCR + EPB * NQ * SCR2 + 1) & ~1;  // 45 unique tangent entries per point
  static constexpr int A_STRIDE = NQ * 45;
  static constexpr int K_STRIDE = 576;                  // K staging per element, over the whole float2 region
  static constexpr int N_F2_USE = F_A + EPB * A_STRIDE;
  static constexpr int N_F2 = N_F2_USE > EPB * K_STRIDE ? N_F2_USE : EPB * K_STRIDE;
  static constexpr size_t BYTES = sizeof(double) * N_DOUBLE + sizeof(float2) * N_F2 + sizeof(int) * EPB * 8 + 16;
};

// 24 threads per element: thread (a, i) owns row (a, i) and the node blocks
// b = a, a+1, a+2, a+3 (mod 8), plus b = a+4 for a < 4 -- a circulant cover of
// the 36 symmetric node pairs, 4 or 5 blocks per row, the other half of K_e
// mirrored in the staging.  Each thread forms the one tangent vector of its row
// and holds 15 accumulators, which fits 4 CTAs (24 warps) on an SM: the df64
// chains are latency-bound, and twice the warps of a 12-thread-per-element
// layout (rows paired as in mech_hex8_sym_kernel) cut the kernel time by 21%.
// One CTA-sized tile of EPB elements (thread (tx, ty): row node and component
// tx, element ty), shared by the kernel below and the single-launch kernel of
// mixed element blocks (which stages without the bulk copy: BULK = false).
template <class Model, int EPB, bool WANT_R, bool WANT_K, bool BULK = true>
__device__ __forceinline__ void hex8_df64_tile(const ElemArgs& g, unsigned tile, int tx, int ty,
                                               unsigned char* smem_raw) {
  constexpr int NQ = 8, TPE = 24, NS = Model::NS, SCR = Model::SCR, SCR2 = Model::SCR2;
  using S = Hex8Df64Smem<Model, EPB>;
  double* dbase = reinterpret_cast<double*>(smem_raw);
  double* s_ref = dbase + S::D_REF;
  float2* fb = reinterpret_cast<float2*>(dbase + S::N_DOUBLE);
  int* s_conn_all = reinterpret_cast<int*>(fb + S::N_F2);

  const int tid = ty * TPE + tx, nthr = EPB * TPE;
  const int64_t e0 = int64_t(tile) * EPB;
  const int64_t e = e0 + ty;
  const bool live = e < g.ne;
  double* s_x = dbase + S::D_X + ty * 24;
  double* s_u = dbase + S::D_U + ty * 24;
  const float2* s_dNX = fb + S::F_DNX + ty * S::DNXS;
  const float2* s_P = fb + S::F_P + ty * NQ * 9;
  const float2* s_scr = fb + S::F_SCR + ty * NQ * SCR2;
  float2* s_A = fb + S::F_A + ty * S::A_STRIDE;
  int* s_conn = s_conn_all + ty * 8;

  {
    const int64_t left = g.ne - e0;
    stage_hex8_tables(g.ref, s_ref, g.conn + e0 * 8, left < EPB ? int(left) : EPB, s_conn_all,
                      reinterpret_cast<uint64_t*>(s_conn_all + EPB * 8), tid, nthr, g.wait_err, g.wait_budget,
                      BULK);
  }
  if (live) {
    const int a = tx / 3, d = tx % 3;
    s_x[tx] = __ldg(&g.coords[int64_t(s_conn[a]) * 3 + d]);
    s_u[tx] = __ldg(&g.U[int64_t(s_conn[a]) * 3 + d]);
  }
  __syncthreads();
  if (tid < EPB * NQ) {  // per-point map and constitutive update, native FP64, full warps
    const int el = tid / NQ, q = tid % NQ;
    const int64_t ep = e0 + el;
    if (ep < g.ne) {
      const double* px = dbase + S::D_X + el * 24;
      const double* pu = dbase + S::D_U + el * 24;
      double dNX[24];
      const double jxw = map_point<1, double>(s_ref, q, px, dNX, nullptr);
      double gu[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double s = 0;
#pragma unroll
          for (int a = 0; a < 8; ++a) s = fma(pu[a * 3 + i], dNX[a * 3 + j], s);
          gu[i][j] = s;
        }
      float2* pdNX = fb + S::F_DNX + el * S::DNXS;
#pragma unroll
      for (int m = 0; m < 24; ++m) pdNX[q * 24 + m] = df64_split(dNX[m]);  // dNX dies before the model
      const double* so = NS ? g.state_old + (ep * NQ + q) * NS : nullptr;
      double* sn = (NS && g.state_new) ? g.state_new + (ep * NQ + q) * NS : nullptr;
      double P9[9], scr[SCR];
      Model::point(g.props, gu, jxw, so, sn, P9, scr);
      float2* pP = fb + S::F_P + el * NQ * 9;
      float2* pscr = fb + S::F_SCR + el * NQ * SCR2;
#pragma unroll
      for (int m = 0; m < 9; ++m) pP[q * 9 + m] = df64_split(P9[m]);
      Model::split_scratch(scr, pscr + q * SCR2);
    }
  }
  __syncthreads();
  if (WANT_K && live) {
    for (int w = tx; w < NQ * 45; w += TPE) {
      const int q = w / 45;
      int r1, r2;
      sym_pair(w - q * 45, r1, r2);
      s_A[w] = Model::aentry_df64(s_scr + q * SCR2, r1 / 3, r1 % 3, r2 / 3, r2 % 3);
    }
  }
  __syncthreads();

  const int a = tx / 3, i = tx % 3;
  const bool fifth = a < 4;
  const int r1v[3] = {3 * i, 3 * i + 1, 3 * i + 2};
  const float2 z = make_float2(0.f, 0.f);
  float2 K[15];
#pragma unroll
  for (int c = 0; c < 15; ++c) K[c] = z;
  float2 R = z;
  if (live) {
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      const float2* dNX = s_dNX + q * 24;
      const float2 g0 = dNX[a * 3], g1 = dNX[a * 3 + 1], g2 = dNX[a * 3 + 2];
      if (WANT_R) {
        const float2* P = s_P + q * 9 + i * 3;
        R = df64_dot3_acc(R, g0, P[0], g1, P[1], g2, P[2]);
      }
      if (WANT_K) {
        const float2* Aq = s_A + q * 45;
        float2 t[9];
#pragma unroll
        for (int kl = 0; kl < 9; ++kl)
          t[kl] = df64_dot3(g0, Aq[sym_index(r1v[0], kl)], g1, Aq[sym_index(r1v[1], kl)], g2,
                            Aq[sym_index(r1v[2], kl)]);
#pragma unroll
        for (int d = 0; d < 5; ++d) {
          if (d == 4 && !fifth) break;
          const int b = (a + d) & 7;
          const float2 h0 = dNX[b * 3], h1 = dNX[b * 3 + 1], h2 = dNX[b * 3 + 2];
#pragma unroll
          for (int k = 0; k < 3; ++k)
            K[d * 3 + k] = df64_dot3_acc(K[d * 3 + k], t[k * 3], h0, t[k * 3 + 1], h1, t[k * 3 + 2], h2);
        }
      }
    }
  }
  // the residual leaves as one double: hi + lo of a normalised pair is exact in FP64
  if (WANT_R && live) static_cast<double*>(g.Re)[e * 24 + tx] = widen(R.x) + widen(R.y);
  __syncthreads();  // the whole float2 region is reused for the K staging below
  if (WANT_K && live) {
    float2* Ks = fb + ty * S::K_STRIDE;  // 576 double-float entries, KE_NODE_ROWS layout
#pragma unroll
    for (int d = 0; d < 5; ++d) {
      if (d == 4 && !fifth) break;
      const int b = (a + d) & 7;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        Ks[((a * 3 + i) * 3 + k) * 8 + b] = K[d * 3 + k];
        if (d) Ks[((b * 3 + k) * 3 + i) * 8 + a] = K[d * 3 + k];
      }
    }
  }
  if (WANT_K) {
    __syncthreads();
    constexpr int PER = 576 / 2;
    const int64_t left = g.ne - e0;
    const int nlive = left < EPB ? int(left) : EPB;
    double2* dst = reinterpret_cast<double2*>(static_cast<double*>(g.Ke) + e0 * 576);
    const double* src = reinterpret_cast<const double*>(fb);
    for (int idx = tid; idx < nlive * PER; idx += nthr) {
      const int el = idx / PER, off = idx - el * PER;
      dst[idx] = *reinterpret_cast<const double2*>(src + el * S::K_STRIDE + off * 2);
    }
  }
}

template <class Model, int EPB, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(EPB * 24, 4) mech_hex8_df64_kernel(ElemArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  hex8_df64_tile<Model, EPB, WANT_R, WANT_K>(g, blockIdx.x, threadIdx.x, threadIdx.y, smem_raw);
}

// ---------------------------------------------------------------------------
// Warp-specialised, persistent form of the FP64 hex8 kernel (the default).
//
// The per-point phase (isoparametric map and constitutive update in native
// FP64, then the double-float splits of the gradients, the stress and the
// tangent scratch) and the double-float work of K_e and R_e (the 45 unique
// tangent entries per point, the contraction) run on different warps of one
// CTA and on different tiles of 16 elements: while 12 consumer warps work on
// tile t, 4 producer warps (one per SM sub-partition, so that every FP64 unit
// of the SM carries a share of the point phase) prepare tile t+1 in the other
// half of a double-buffered shared-memory stage.  One CTA per SM takes the
// tiles blockIdx.x, blockIdx.x + gridDim.x, ...  The hand-over uses named
// barriers: FULL[b] (producers arrive, consumers wait) and EMPTY[b] (consumers
// arrive after their last read of stage b, producers wait before refilling it).
// Every warp of a role runs the same tile sequence and reaches every barrier,
// so each barrier generation completes with exactly NTHR threads.  The
// arithmetic is that of hex8_df64_tile, operation for operation, so both give
// bitwise the same workspace.
// ---------------------------------------------------------------------------
namespace ws {
constexpr int EPB = 16, NQ = 8;
constexpr int PROD_WARPS = 4, CONS_WARPS = 12;
constexpr int NPROD = 32 * PROD_WARPS;  // one thread per quadrature point of the tile
constexpr int NCONS = 32 * CONS_WARPS;  // one thread per row of K_e of the tile
constexpr int NTHR = NPROD + NCONS;
static_assert(NPROD == EPB * NQ && NCONS == EPB * 24, "tile shape");
// named barrier ids (0 is __syncthreads)
constexpr int BAR_FULL = 1;   // 1, 2: stage b filled
constexpr int BAR_EMPTY = 3;  // 3, 4: stage b consumed
constexpr int BAR_PROD = 5;   // producers only
constexpr int BAR_CONS = 6;   // consumers only
constexpr int REF_BYTES = ((RefLayout<1>::SIZE * 8 + 15) / 16) * 16;

// shared memory (bytes): reference tables, then two stages of
template <class Model>
struct Layout {
  static constexpr int X = 0;                           // double [EPB][24] coordinates
  static constexpr int U = X + EPB * 24 * 8;            // double [EPB][24] displacements
  static constexpr int DNXS = NQ * 24;                  // float2 [EPB][NQ][24] spatial gradients
  static constexpr int DNX = U + EPB * 24 * 8;
  static constexpr int P = DNX + EPB * DNXS * 8;        // float2 [EPB][NQ][9] JxW P
  static constexpr int SCR = P + EPB * NQ * 9 * 8;      // float2 [EPB][NQ][SCR2] tangent scratch
  static constexpr int A = SCR + EPB * NQ * Model::SCR2 * 8;  // float2 [EPB][NQ][45] JxW A, unique entries
  static constexpr int STAGE = ((A + EPB * NQ * 45 * 8) + 15) / 16 * 16;
  static constexpr int K_BYTES = EPB * 576 * 8;         // K_e staging over a consumed stage
  static_assert(K_BYTES <= STAGE, "stage layout");
  static constexpr int SMEM = REF_BYTES + 2 * STAGE;
};

__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void named_arrive(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
}  // namespace ws

template <class Model, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(ws::NTHR, 1) mech_hex8_df64_ws_kernel(ElemArgs g) {
  using namespace ws;
  using Lay = Layout<Model>;
  constexpr int NS = Model::NS, SCR = Model::SCR, SCR2 = Model::SCR2;
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_ref = reinterpret_cast<double*>(smem);
  const int tid = threadIdx.x;
  for (int i = tid; i < RefLayout<1>::SIZE; i += NTHR) s_ref[i] = g.ref[i];
  __syncthreads();
  const int64_t ntiles = (g.ne + EPB - 1) / EPB;

  if (tid < NPROD) {
    // ---- producers: thread (el, q) owns quadrature point q of element el ----
    const int el = tid >> 3, q = tid & 7;
    for (int k = 0;; ++k) {
      const int64_t tile = blockIdx.x + int64_t(k) * gridDim.x;
      if (tile >= ntiles) break;
      const int buf = k & 1;
      unsigned char* st = smem + REF_BYTES + buf * Lay::STAGE;
      if (k >= 2) named_sync(BAR_EMPTY + buf, NTHR);  // the consumers are done with tile k-2
      const int64_t e = tile * EPB + el;
      const bool live = e < g.ne;
      double* s_x = reinterpret_cast<double*>(st + Lay::X) + el * 24;
      double* s_u = reinterpret_cast<double*>(st + Lay::U) + el * 24;
      if (live) {
        const int64_t node = g.conn[e * 8 + q];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          s_x[q * 3 + d] = __ldg(&g.coords[node * 3 + d]);
          s_u[q * 3 + d] = __ldg(&g.U[node * 3 + d]);
        }
      }
      named_sync(BAR_PROD, NPROD);
      if (live) {
        double dNX[24];
        const double jxw = map_point<1, double>(s_ref, q, s_x, dNX, nullptr);
        double gu[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            double sum = 0;
#pragma unroll
            for (int a = 0; a < 8; ++a) sum = fma(s_u[a * 3 + i], dNX[a * 3 + j], sum);
            gu[i][j] = sum;
          }
        const int pt = el * NQ + q;
        float2* pdNX = reinterpret_cast<float2*>(st + Lay::DNX) + el * Lay::DNXS + q * 24;
#pragma unroll
        for (int m = 0; m < 24; ++m) pdNX[m] = df64_split(dNX[m]);  // dNX dies before the model
        const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
        double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
        double P9[9], scr[SCR];
        Model::point(g.props, gu, jxw, so, sn, P9, scr);
        float2* pP = reinterpret_cast<float2*>(st + Lay::P) + pt * 9;
#pragma unroll
        for (int m = 0; m < 9; ++m) pP[m] = df64_split(P9[m]);
        Model::split_scratch(scr, reinterpret_cast<float2*>(st + Lay::SCR) + pt * SCR2);
      }
      named_arrive(BAR_FULL + buf, NTHR);
    }
    return;
  }

  // ---- consumers: thread (el, tx) owns row tx = (a, i) of element el's K_e (a warp
  // spans fewer than two elements, so its gradient loads touch few distinct addresses) ----
  const int c = tid - NPROD, el = c / 24, tx = c - el * 24;
  const int a = tx / 3, i = tx % 3;
  const bool fifth = a < 4;
  const int r1v[3] = {3 * i, 3 * i + 1, 3 * i + 2};
  const float2 z = make_float2(0.f, 0.f);
  for (int k = 0;; ++k) {
    const int64_t tile = blockIdx.x + int64_t(k) * gridDim.x;
    if (tile >= ntiles) break;
    const int buf = k & 1;
    unsigned char* st = smem + REF_BYTES + buf * Lay::STAGE;
    named_sync(BAR_FULL + buf, NTHR);  // tile k is in stage buf
    const int64_t e0 = tile * EPB, e = e0 + el;
    const bool live = e < g.ne;
    const float2* s_dNX = reinterpret_cast<const float2*>(st + Lay::DNX) + el * Lay::DNXS;
    const float2* s_P = reinterpret_cast<const float2*>(st + Lay::P) + el * NQ * 9;
    const float2* s_scr = reinterpret_cast<const float2*>(st + Lay::SCR) + el * NQ * SCR2;
    float2* s_A = reinterpret_cast<float2*>(st + Lay::A) + el * NQ * 45;
    if (WANT_K) {
      if (live)
        for (int w = tx; w < NQ * 45; w += 24) {
          const int q = w / 45;
          int r1, r2;
          sym_pair(w - q * 45, r1, r2);
          s_A[w] = Model::aentry_df64(s_scr + q * SCR2, r1 / 3, r1 % 3, r2 / 3, r2 % 3);
        }
      named_sync(BAR_CONS, NCONS);
    }
    float2 K[15];
#pragma unroll
    for (int cc = 0; cc < 15; ++cc) K[cc] = z;
    float2 R = z;
    if (live) {
#pragma unroll 1
      for (int q = 0; q < NQ; ++q) {
        const float2* dNX = s_dNX + q * 24;
        const float2 g0 = dNX[a * 3], g1 = dNX[a * 3 + 1], g2 = dNX[a * 3 + 2];
        if (WANT_R) {
          const float2* P = s_P + q * 9 + i * 3;
          R = df64_dot3_acc(R, g0, P[0], g1, P[1], g2, P[2]);
        }
        if (WANT_K) {
          const float2* Aq = s_A + q * 45;
          float2 t[9];
#pragma unroll
          for (int kl = 0; kl < 9; ++kl)
            t[kl] = df64_dot3(g0, Aq[sym_index(r1v[0], kl)], g1, Aq[sym_index(r1v[1], kl)], g2,
                              Aq[sym_index(r1v[2], kl)]);
#pragma unroll
          for (int d = 0; d < 5; ++d) {
            if (d == 4 && !fifth) break;
            const int b = (a + d) & 7;
            const float2 h0 = dNX[b * 3], h1 = dNX[b * 3 + 1], h2 = dNX[b * 3 + 2];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
              K[d * 3 + kk] = df64_dot3_acc(K[d * 3 + kk], t[kk * 3], h0, t[kk * 3 + 1], h1, t[kk * 3 + 2], h2);
          }
        }
      }
    }
    if (WANT_R && live) static_cast<double*>(g.Re)[e * 24 + tx] = widen(R.x) + widen(R.y);
    if (WANT_K) {
      named_sync(BAR_CONS, NCONS);  // every consumer is done reading stage buf: stage K_e over it
      if (live) {
        float2* Ks = reinterpret_cast<float2*>(st) + el * 576;  // KE_NODE_ROWS layout
#pragma unroll
        for (int d = 0; d < 5; ++d) {
          if (d == 4 && !fifth) break;
          const int b = (a + d) & 7;
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            Ks[((a * 3 + i) * 3 + kk) * 8 + b] = K[d * 3 + kk];
            if (d) Ks[((b * 3 + kk) * 3 + i) * 8 + a] = K[d * 3 + kk];
          }
        }
      }
      named_sync(BAR_CONS, NCONS);
      const int64_t left = g.ne - e0;
      const int nlive = left < EPB ? int(left) : EPB;
      double2* dst = reinterpret_cast<double2*>(static_cast<double*>(g.Ke) + e0 * 576);
      const double2* src = reinterpret_cast<const double2*>(st);
      for (int idx = c; idx < nlive * 288; idx += NCONS) dst[idx] = src[idx];
    }
    named_arrive(BAR_EMPTY + buf, NTHR);  // stage buf may be refilled
  }
}

}  // namespace fec
