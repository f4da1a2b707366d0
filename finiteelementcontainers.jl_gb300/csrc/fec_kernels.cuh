// fec_kernels.cuh -- sm_103a kernels of the assembly path.
//
// Two kernel families run per fec_assemble call:
//
//  1. element kernels (one launch per element block, as foreach_block in
//     src/Utils.jl:171-189 launches _assemble_block! per block): a CTA holds
//     EPB elements; each element is served by TPE = NDOF*CSPLIT threads, one
//     (row, column-chunk) of the element matrix each.  The connectivity and the
//     nodal coordinates/field are gathered once per element into shared memory;
//     the quadrature-point kinematics (isoparametric map, deformation gradient)
//     and the constitutive update are computed once per point and shared; every
//     thread then accumulates its row of K_e and R_e over the points in q order
//     (src/assemblers/Assemblers.jl:418-431).  K_e is written row-major
//     (K_e[r][c] = dR_r/du_c) and R_e next to it, into element-ordered storage:
//     the same element-slot layout the reference fills in
//     src/assemblers/Assemblers.jl:109-124 (there column-major, i.e. transposed).
//
//  2. the node gather (one warp per mesh node): walks the node's adjacent
//     elements in increasing element order, reads the rows of K_e/R_e that
//     belong to the node (contiguous, coalesced), and adds each value to its
//     CSC position in a shared-memory accumulator.  Each CSC entry therefore
//     receives its element contributions in increasing element order -- the
//     order SparseArrays.sparse! combines the reference's element-ordered COO
//     entries (src/assemblers/SparsityPatterns.jl:301-308) -- with no atomics,
//     so results are bitwise reproducible.  The node's CSC columns are
//     contiguous in nzval (unknowns are numbered node-major), so the final
//     write is coalesced too.  The residual over unknowns is produced in the
//     same pass (residual(asm), src/assemblers/Assemblers.jl:347-371).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>
#include "fec_df64.cuh"

namespace fec {

// ---------------------------------------------------------------------------
// element traits
// ---------------------------------------------------------------------------
template <int ET> struct Elem;
template <> struct Elem<1> { static constexpr int DIM = 3, NNPE = 8, NQ = 8; };    // HEX8
template <> struct Elem<2> { static constexpr int DIM = 2, NNPE = 4, NQ = 4; };    // QUAD4
template <> struct Elem<6> { static constexpr int DIM = 3, NNPE = 4, NQ = 1; };    // TET4
template <> struct Elem<7> { static constexpr int DIM = 3, NNPE = 10, NQ = 4; };   // TET10
template <> struct Elem<8> { static constexpr int DIM = 3, NNPE = 27, NQ = 27; };  // HEX27

// Reference-element tables, packed: N[q][a], dN[q][a][k], w[q] (doubles).
template <int ET> struct RefLayout {
  using E = Elem<ET>;
  static constexpr int N_OFF = 0;
  static constexpr int DN_OFF = E::NQ * E::NNPE;
  static constexpr int W_OFF = DN_OFF + E::NQ * E::NNPE * E::DIM;
  static constexpr int SIZE = W_OFF + E::NQ;
};

struct ElemArgs {
  const int32_t* conn;      // block connectivity, 0-based, conn[e*NNPE + a]
  int64_t ne;               // elements in the block
  const double* coords;     // coords[node*DIM + d]
  const double* U;          // U[node*NF + f]
  const double* ref;        // reference tables (RefLayout)
  double props[8];
  const double* state_old;  // block base, (NS, NQ, NE) column-major
  double* state_new;
  void* Ke;                 // block base, Real[ne][NDOF][NDOF]
  void* Re;                 // block base, Real[ne][NDOF]
  const void* closure;      // learned-closure data (ClosureArgs) for the physics that uses one
  const void* affine;       // hex8 blocks of translated elements: the constant operand table (or null)
  int* wait_err;            // set to 1 by a bounded wait that gave up (device flag; may be null)
  long long wait_budget;    // SM clocks a bounded wait allows before giving up (0: the default, ~1 s)
  int ke_pairs;             // the element kernel writes KE_PAIRS (FP64 hex8 tensor-core, FP64 hex27 kernels)
};

// ---------------------------------------------------------------------------
// Element workspace entries.  FP32-element kernels store floats.  FP64 kernels
// store double-float pairs (hi, lo), 8 bytes like a double: the df64 kernel
// produces them directly, the others split their FP64 results.  The node gather
// then accumulates in compensated FP32 on the FP32 pipes and touches the FP64
// pipe once per assembled entry (the GB300's FP64 pipe is 1/64 of its FP32
// rate and occupies a whole warp-instruction slot however few lanes are active).
// ---------------------------------------------------------------------------
template <typename Real> struct WS;
template <> struct WS<double> {
  using T = float2;
  __device__ static T from(double v) { return df64_split(v); }
};
template <> struct WS<float> {
  using T = float;
  __device__ static T from(float v) { return v; }
};
// Element residuals are stored in the arithmetic's own type: double in the FP64
// variant (formed in native FP64 and summed in FP64 by the node gather, so the
// residual keeps FP64 accuracy), float in the FP32-element variant.  RE<W> maps
// the gather's matrix-entry type to it.
template <typename W> struct RE;
template <> struct RE<float2> { using T = double; };
template <> struct RE<float> { using T = float; };

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double det3(const double J[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

// Isoparametric map at one point, always in FP64: J = X_el dN_xi, JxW = det(J) w,
// dN_X = dN_xi J^{-1}.  Writes dN_X (as Real) and returns JxW; Xq optional.
template <int ET, typename Real>
__device__ __forceinline__ double map_point(const double* __restrict__ s_ref, int q, const double* __restrict__ s_x,
                                            Real* __restrict__ dNX, double* Xq) {
  using E = Elem<ET>;
  using L = RefLayout<ET>;
  constexpr int D = E::DIM, A = E::NNPE;
  const double* dN = s_ref + L::DN_OFF + q * A * D;
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int a = 0; a < A; ++a)
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
      for (int k = 0; k < D; ++k) J[d][k] = fma(s_x[a * D + d], dN[a * D + k], J[d][k]);
  double Ji[3][3];
  double det;
  if (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double r = 1.0 / det;
    Ji[0][0] = J[1][1] * r; Ji[0][1] = -J[0][1] * r;
    Ji[1][0] = -J[1][0] * r; Ji[1][1] = J[0][0] * r;
  } else {
    det = det3(J);
    const double r = 1.0 / det;
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * r;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * r;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * r;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  }
#pragma unroll
  for (int a = 0; a < A; ++a)
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double s = 0;
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(dN[a * D + k], Ji[k][d], s);
      dNX[a * D + d] = Real(s);
    }
  if (Xq) {
    const double* N = s_ref + L::N_OFF + q * A;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double s = 0;
#pragma unroll
      for (int a = 0; a < A; ++a) s = fma(N[a], s_x[a * D + d], s);
      Xq[d] = s;
    }
  }
  return det * s_ref[L::W_OFF + q];
}

// FP32 map of a 3-D point from FP64-differenced coordinates xd[a] = x[a] - x[0]
// (J = sum_a xd_a (x) dN_a, since sum_a dN_a = 0); falls back to the FP64 map
// for distorted elements (Hadamard ratio |det J| / prod |J col| < 0.25).
// Returns JxW.
template <int ET>
__device__ __forceinline__ float map_point_mixed(const double* __restrict__ s_ref, const float* __restrict__ s_reff,
                                                 int q, const double* __restrict__ x, const float* __restrict__ xd,
                                                 float* __restrict__ dNX) {
  using E = Elem<ET>;
  using L = RefLayout<ET>;
  constexpr int A = E::NNPE;
  static_assert(E::DIM == 3, "3-D elements");
  const float* dN = s_reff + L::DN_OFF + q * A * 3;
  float J[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
  for (int a = 1; a < A; ++a)
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
  if (!(fabsf(det) >= 0.25f * sqrtf(n0 * n1 * n2))) return float(map_point<ET, float>(s_ref, q, x, dNX, nullptr));
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
  for (int a = 0; a < A; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      dNX[a * 3 + d] = fmaf(dN[a * 3], Ji[0][d], fmaf(dN[a * 3 + 1], Ji[1][d], dN[a * 3 + 2] * Ji[2][d]));
  return det * s_reff[L::W_OFF + q];
}

// Copy the reference tables and gather X (and U) of each element of the CTA
// into shared memory.  Threads of element slot ty use tx = 0..TPE-1; slots
// ty >= EPB (threads past EPB * TPE in a CTA of NTHR threads) only take part in
// the barriers, and the caller passes them an element index e >= g.ne.
template <int ET, int NF, int EPB, int TPE, int NTHR = EPB * TPE>
__device__ __forceinline__ void stage_element(const ElemArgs& g, int64_t e, int tx, int ty, double* s_ref, int* s_conn,
                                              double* s_x, double* s_u) {
  using E = Elem<ET>;
  constexpr int D = E::DIM, A = E::NNPE;
  static_assert(NTHR >= EPB * TPE, "NTHR covers the element slots");
  const int tid = ty * TPE + tx;
  if (NTHR == EPB * TPE || tid < EPB * TPE)
    for (int i = tid; i < RefLayout<ET>::SIZE; i += EPB * TPE) s_ref[i] = g.ref[i];
  const bool live = e < g.ne;
  if (live)
    for (int a = tx; a < A; a += TPE) s_conn[a] = g.conn[e * A + a];
  __syncthreads();
  if (live) {
    for (int i = tx; i < A * D; i += TPE) s_x[i] = __ldg(&g.coords[int64_t(s_conn[i / D]) * D + (i % D)]);
    for (int i = tx; i < A * NF; i += TPE) s_u[i] = __ldg(&g.U[int64_t(s_conn[i / NF]) * NF + (i % NF)]);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Poisson (test/poisson/TestPoissonCommon.jl:75-107):
//   R_q = JxW (grad u . dN_X_a - N_a f(X_q)),  K_q = JxW dN_X_a . dN_X_b
// one thread per element row a.  AFF (FP64 blocks of translated hex8 elements,
// g.affine: the block's spatial gradients [q][a][d] then JxW [q], double): the
// map is the same for every element and is read, only X_q is formed.
// ---------------------------------------------------------------------------
template <int ET, typename Real, int EPB, bool WANT_R, bool WANT_K, bool AFF = false>
__global__ void __launch_bounds__(EPB * Elem<ET>::NNPE) poisson_element_kernel(ElemArgs g) {
  using E = Elem<ET>;
  using L = RefLayout<ET>;
  constexpr int D = E::DIM, A = E::NNPE, NQ = E::NQ, TPE = A;
  __shared__ double s_ref[L::SIZE];
  __shared__ int s_conn_all[EPB][A];
  __shared__ double s_x_all[EPB][A * D];
  __shared__ double s_u_all[EPB][A];
  __shared__ Real s_dNX_all[EPB][NQ][A * D];
  __shared__ Real s_jxw_all[EPB][NQ];
  __shared__ Real s_gu_all[EPB][NQ][D];
  __shared__ Real s_f_all[EPB][NQ];

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t e = int64_t(blockIdx.x) * EPB + ty;
  stage_element<ET, 1, EPB, TPE>(g, e, tx, ty, s_ref, s_conn_all[ty], s_x_all[ty], s_u_all[ty]);
  const bool live = e < g.ne;
  static_assert(!AFF || (ET == 1 && sizeof(Real) == 8), "block gradients: FP64 hex8");
  if (live) {
    for (int q = tx; q < NQ; q += TPE) {
      double Xq[3];
      Real* dNX = s_dNX_all[ty][q];
      double jxw;
      if constexpr (AFF) {
        const double* tg = static_cast<const double*>(g.affine);
#pragma unroll
        for (int k = 0; k < A * D; ++k) dNX[k] = Real(__ldg(tg + q * A * D + k));
        jxw = __ldg(tg + NQ * A * D + q);
        if (WANT_R) {
          const double* N = s_ref + L::N_OFF + q * A;
          const double* x = s_x_all[ty];
#pragma unroll
          for (int d = 0; d < D; ++d) {
            double s = 0;
#pragma unroll
            for (int a = 0; a < A; ++a) s = fma(N[a], x[a * D + d], s);
            Xq[d] = s;
          }
        }
      } else {
        jxw = map_point<ET, Real>(s_ref, q, s_x_all[ty], dNX, Xq);
      }
      s_jxw_all[ty][q] = Real(jxw);
      if (WANT_R) {
        double f = g.props[0];
#pragma unroll
        for (int d = 0; d < D; ++d) f *= sin(M_PI * Xq[d]);
        s_f_all[ty][q] = Real(jxw * f);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          Real s = 0;
#pragma unroll
          for (int a = 0; a < A; ++a) s = fma(Real(s_u_all[ty][a]), dNX[a * D + d], s);
          s_gu_all[ty][q][d] = s;
        }
      }
    }
  }
  __syncthreads();
  if (!live) return;
  const int a = tx;
  Real Krow[A];
#pragma unroll
  for (int b = 0; b < A; ++b) Krow[b] = 0;
  Real R = 0;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const Real* dNX = s_dNX_all[ty][q];
    const Real w = s_jxw_all[ty][q];
    Real ga[D];
#pragma unroll
    for (int d = 0; d < D; ++d) ga[d] = dNX[a * D + d];
    if (WANT_R) {
      Real s = 0;
#pragma unroll
      for (int d = 0; d < D; ++d) s = fma(s_gu_all[ty][q][d], ga[d], s);
      R = fma(w, s, R);
      R = fma(-Real(s_ref[L::N_OFF + q * A + a]), s_f_all[ty][q], R);
    }
    if (WANT_K) {
#pragma unroll
      for (int d = 0; d < D; ++d) ga[d] *= w;
#pragma unroll
      for (int b = 0; b < A; ++b) {
        Real s = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) s = fma(ga[d], dNX[b * D + d], s);
        Krow[b] += s;
      }
    }
  }
  if (WANT_K) {
    typename WS<Real>::T* Ke = static_cast<typename WS<Real>::T*>(g.Ke) + (e * A + a) * A;
#pragma unroll
    for (int b = 0; b < A; ++b) Ke[b] = WS<Real>::from(Krow[b]);
  }
  if (WANT_R) static_cast<Real*>(g.Re)[e * A + a] = R;
}

// ---------------------------------------------------------------------------
// Constitutive models for the mechanics kernel.  Per quadrature point, point()
// receives grad u (row-major [i][J]) and writes JxW-scaled P (P9[i*3+J]) plus
// what aentries() needs to produce JxW-scaled A_iJkL for one i.
// ---------------------------------------------------------------------------

// A product rounded on its own: never fused into an FMA, so every kernel that
// inlines a constitutive update rounds it alike (the single launch across blocks
// and the per-block kernels give bitwise the same results).
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

// Compressible Neo-Hookean (test/mechanics/TestMechanicsLargeDeformation.jl:17-27)
//   psi = K/2 (1/2 (J-1)^2 - ln J) + G/2 (J^{-2/3} F:F - 3)
//   P = c1 H + c2 (F - I1/3 H),  H = F^{-T}, c1 = K/2 (J^2-J-1), c2 = G J^{-2/3}
//   A_iJkL = a1 H_iJ H_kL + a2 H_iL H_kJ + c2 d_ik d_JL - 2/3 c2 (H_kL F_iJ + F_kL H_iJ)
//   a1 = K/2 (2J-1) J + 2/9 c2 I1,  a2 = I1/3 c2 - c1
struct NeoHookean {
  static constexpr bool USES_CLOSURE = false;
  static constexpr bool USES_TABLE = false;
  static constexpr int NS = 0;
  static constexpr int SCR = 21;  // F(9) H(9) a1 a2 c2
  template <typename Real>
  __device__ static void point(const double* props, Real gu[3][3], Real jxw, const double*, double*, Real* P9,
                               Real* scr) {
    const Real Kb = Real(props[0]), Gs = Real(props[1]);
    Real F[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] = gu[i][j] + (i == j ? Real(1) : Real(0));
    const Real c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    const Real c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    const Real c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    const Real J = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    const Real rJ = Real(1) / J;
    Real H[3][3];
    H[0][0] = c00 * rJ; H[0][1] = c01 * rJ; H[0][2] = c02 * rJ;
    H[1][0] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * rJ;
    H[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * rJ;
    H[1][2] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * rJ;
    H[2][0] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * rJ;
    H[2][1] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * rJ;
    H[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * rJ;
    Real I1 = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) I1 = fma(F[i][j], F[i][j], I1);
    const Real c1 = Real(0.5) * Kb * (J * J - J - Real(1));
    const Real r3 = rcbrt(J);  // J^{-1/3}
    const Real c2 = Gs * r3 * r3;
    const Real I13 = mul_rn(I1, Real(1.0 / 3.0));  // (a multiply: FP64 divisions are long on the FP64 pipe)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P9[i * 3 + j] = jxw * (c1 * H[i][j] + c2 * (F[i][j] - I13 * H[i][j]));
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      scr[i] = F[i / 3][i % 3];
      scr[9 + i] = H[i / 3][i % 3];
    }
    scr[18] = jxw * (Real(0.5) * Kb * (Real(2) * J - Real(1)) * J + Real(2.0 / 9.0) * c2 * I1);
    scr[19] = jxw * (I13 * c2 - c1);
    scr[20] = jxw * c2;
  }
  // JxW A_iJkL
  template <typename Real>
  __device__ static Real aentry(const Real* scr, int i, int J, int k, int L) {
    const Real* F = scr;
    const Real* H = scr + 9;
    Real v = scr[18] * H[i * 3 + J] * H[k * 3 + L] + scr[19] * H[i * 3 + L] * H[k * 3 + J] +
             Real(-2.0 / 3.0) * scr[20] * (H[k * 3 + L] * F[i * 3 + J] + F[k * 3 + L] * H[i * 3 + J]);
    if (i == k && J == L) v += scr[20];
    return v;
  }
  // JxW (A : G)_iJ = sum_kL A_iJkL G_kL for a direction gradient G, without forming A:
  // a1 (H:G) H + a2 H G^T H - 2/3 c2 ((H:G) F + (F:G) H) + c2 G
  template <typename Real>
  __device__ static void action(const Real* scr, const Real G[3][3], Real out[3][3]) {
    const Real* F = scr;
    const Real* H = scr + 9;
    Real hg = 0, fg = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int L = 0; L < 3; ++L) {
        hg = fma(H[k * 3 + L], G[k][L], hg);
        fg = fma(F[k * 3 + L], G[k][L], fg);
      }
    Real M[3][3];  // (G^T H)_LJ
#pragma unroll
    for (int L = 0; L < 3; ++L)
#pragma unroll
      for (int J = 0; J < 3; ++J) M[L][J] = G[0][L] * H[J] + G[1][L] * H[3 + J] + G[2][L] * H[6 + J];
    const Real m23 = Real(-2.0 / 3.0) * scr[20];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int J = 0; J < 3; ++J) {
        const Real hgh = H[i * 3] * M[0][J] + H[i * 3 + 1] * M[1][J] + H[i * 3 + 2] * M[2][J];
        out[i][J] = scr[18] * hg * H[i * 3 + J] + scr[19] * hgh + m23 * (hg * F[i * 3 + J] + fg * H[i * 3 + J]) +
                    scr[20] * G[i][J];
      }
  }
  // df64 form of the scratch: F(9), H(9), a1, a2, c2, -2/3 c2 (all JxW-scaled where scr is)
  static constexpr int SCR2 = 22;
  __device__ static void split_scratch(const double* scr, float2* out) {
#pragma unroll
    for (int m = 0; m < 21; ++m) out[m] = df64_split(scr[m]);
    out[21] = df64_split(-2.0 / 3.0 * scr[20]);
  }
  // An upper bound of max |JxW A_iJkL| from the df64 scratch (hi parts, FP32):
  // (|a1| + |a2|) max|H|^2 + 2 |2/3 c2| max|H| max|F| + |c2|.
  __device__ static float abound(const float2* s) {
    float hm = 0.f, fm = 0.f;
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      fm = fmaxf(fm, fabsf(s[m].x));
      hm = fmaxf(hm, fabsf(s[9 + m].x));
    }
    return (fabsf(s[18].x) + fabsf(s[19].x)) * hm * hm + 2.f * fabsf(s[21].x) * hm * fm + fabsf(s[20].x);
  }
  // JxW A_iJkL in df64
  __device__ static float2 aentry_df64(const float2* s, int i, int J, int k, int L) {
    const float2* F = s;
    const float2* H = s + 9;
    float2 v = df64_mul(s[18], df64_mul(H[i * 3 + J], H[k * 3 + L]));
    v = df64_fma(s[19], df64_mul(H[i * 3 + L], H[k * 3 + J]), v);
    const float2 t = df64_fma(H[k * 3 + L], F[i * 3 + J], df64_mul(F[k * 3 + L], H[i * 3 + J]));
    v = df64_fma(s[21], t, v);
    if (i == k && J == L) v = df64_add(v, s[20]);
    return v;
  }
  // out[J*9 + k*3 + L] = JxW A_iJkL
  template <typename Real>
  __device__ static void aentries(const Real* scr, int i, Real* out) {
    const Real* F = scr;
    const Real* H = scr + 9;
    const Real a1 = scr[18], a2 = scr[19], c2 = scr[20];
    const Real m23 = Real(-2.0 / 3.0) * c2;
#pragma unroll
    for (int J = 0; J < 3; ++J)
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int L = 0; L < 3; ++L) {
          Real v = a1 * H[i * 3 + J] * H[k * 3 + L] + a2 * H[i * 3 + L] * H[k * 3 + J] +
                   m23 * (H[k * 3 + L] * F[i * 3 + J] + F[k * 3 + L] * H[i * 3 + J]);
          if (i == k && J == L) v += c2;
          out[J * 9 + k * 3 + L] = v;
        }
  }
};

// J2 small-strain plasticity with linear isotropic hardening: radial return and
// the consistent tangent (Simo & Hughes 1998, Box 3.2).  props = {E, nu, sy, H};
// state (7) = plastic strain (xx, yy, zz, yz, xz, xy) + equivalent plastic strain.
struct J2 {
  static constexpr bool USES_CLOSURE = false;
  static constexpr bool USES_TABLE = false;
  static constexpr int NS = 7;
  static constexpr int SCR = 13;  // n(9) kap' 2mu th' 2mu thb' (unused)
  // props: E, nu, sigma_y, H, then the constants derived from them, filled by the
  // library (fec_physics_set, fec_j2_points) so that no point divides for them:
  // mu, kappa, 1 / (2 mu + 2/3 H), 1 / (1 + H / (3 mu)).
  __host__ __device__ static void fill_derived(double* p) {
    const double E = p[0], nu = p[1], H = p[3];
    const double mu = E / (2 * (1 + nu)), lam = E * nu / ((1 + nu) * (1 - 2 * nu));
    p[4] = mu;
    p[5] = lam + 2.0 / 3.0 * mu;
    p[6] = 1.0 / (2 * mu + 2.0 / 3.0 * H);
    p[7] = 1.0 / (1.0 + H / (3 * mu));
  }
  // Arithmetic in Real: double for the FP64 variant, float for the FP32-element
  // variant; the state is accumulated in double either way.  One reciprocal of
  // |s| for the flow direction and the factors (FP64 divisions are long
  // sequences on the FP64 pipe).
  template <typename Real>
  __device__ static void point(const double* props, Real gu[3][3], Real jxw, const double* st_old, double* st_new,
                               Real* P9, Real* scr) {
    using C = Real;
    const C sy = C(props[2]), Hh = C(props[3]);
    const C mu = C(props[4]), kap = C(props[5]), rdg = C(props[6]), thb0 = C(props[7]);
    C eps[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) eps[i][j] = C(0.5) * (C(gu[i][j]) + C(gu[j][i]));
    const C ep[3][3] = {{C(st_old[0]), C(st_old[5]), C(st_old[4])},
                        {C(st_old[5]), C(st_old[1]), C(st_old[3])},
                        {C(st_old[4]), C(st_old[3]), C(st_old[2])}};
    const C eqps_old = C(st_old[6]);
    C ee[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) ee[i][j] = eps[i][j] - ep[i][j];
    const C tr = ee[0][0] + ee[1][1] + ee[2][2], tr3 = mul_rn(tr, C(1.0 / 3.0));
    C s[3][3];
    C sn2 = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        s[i][j] = 2 * mu * (ee[i][j] - (i == j ? tr3 : C(0.0)));
        sn2 += s[i][j] * s[i][j];
      }
    const C snorm = sqrt(sn2);
    const C sq23 = C(sqrt(2.0 / 3.0));
    const C f = snorm - sq23 * (sy + Hh * eqps_old);
    C dgam = 0, th = 1, thb = 0;
    C n[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (f > 0) {
      dgam = mul_rn(f, rdg);
      const C rsn = C(1.0) / snorm;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) n[i][j] = mul_rn(s[i][j], rsn);
      th = C(1.0) - mul_rn(2 * mu * dgam, rsn);
      thb = thb0 - (C(1.0) - th);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        P9[i * 3 + j] = Real(C(jxw) * (s[i][j] - 2 * mu * dgam * n[i][j] + (i == j ? kap * tr : C(0.0))));
    if (st_new) {
      st_new[0] = st_old[0] + double(dgam * n[0][0]);
      st_new[1] = st_old[1] + double(dgam * n[1][1]);
      st_new[2] = st_old[2] + double(dgam * n[2][2]);
      st_new[3] = st_old[3] + double(dgam * n[1][2]);
      st_new[4] = st_old[4] + double(dgam * n[0][2]);
      st_new[5] = st_old[5] + double(dgam * n[0][1]);
      st_new[6] = st_old[6] + double(sq23 * dgam);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) scr[i] = Real(n[i / 3][i % 3]);
    // (rounded on their own: the tangent's consumers subtract them, and a product
    // fused there in one kernel but not in another would differ in the last bit)
    scr[9] = Real(mul_rn(C(jxw), kap));
    scr[10] = Real(mul_rn(mul_rn(C(jxw) * 2, mu), th));
    scr[11] = Real(mul_rn(mul_rn(C(jxw) * 2, mu), thb));
    scr[12] = 0;
  }
  template <typename Real>
  __device__ static Real aentry(const Real* scr, int i, int J, int k, int L) {
    const Real dij = (i == J) ? Real(1) : Real(0), dkl = (k == L) ? Real(1) : Real(0);
    const Real isym = Real(0.5) * (Real((i == k) && (J == L)) + Real((i == L) && (J == k)));
    return scr[9] * dij * dkl + scr[10] * (isym - dij * dkl / Real(3)) - scr[11] * scr[i * 3 + J] * scr[k * 3 + L];
  }
  // JxW (A : G)_iJ = kap' tr(G) d_iJ + 2 mu th' (sym(G) - tr(G)/3 I)_iJ - 2 mu thb' n_iJ (n : G)
  template <typename Real>
  __device__ static void action(const Real* scr, const Real G[3][3], Real out[3][3]) {
    const Real* n = scr;
    const Real tr = G[0][0] + G[1][1] + G[2][2];
    Real ng = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int L = 0; L < 3; ++L) ng = fma(n[k * 3 + L], G[k][L], ng);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int J = 0; J < 3; ++J) {
        const Real d = i == J ? Real(1) : Real(0);
        out[i][J] = scr[9] * tr * d + scr[10] * (Real(0.5) * (G[i][J] + G[J][i]) - tr / Real(3) * d) -
                    scr[11] * n[i * 3 + J] * ng;
      }
  }
  // df64 form: n(9), c_a = kap' - mt'/3 (d_iJ d_kL), c_b = mt'/2 (each I_sym term), mb'
  static constexpr int SCR2 = 12;
  __device__ static void split_scratch(const double* scr, float2* out) {
#pragma unroll
    for (int m = 0; m < 9; ++m) out[m] = df64_split(scr[m]);
    out[9] = df64_split(scr[9] - scr[10] / 3.0);
    out[10] = df64_split(0.5 * scr[10]);
    out[11] = df64_split(scr[11]);
  }
  // An upper bound of max |C_iJkL| from the df64 scratch: |mb'| max|n|^2 + |c_a| + 2 |c_b|.
  __device__ static float abound(const float2* s) {
    float nm = 0.f;
#pragma unroll
    for (int m = 0; m < 9; ++m) nm = fmaxf(nm, fabsf(s[m].x));
    return fabsf(s[11].x) * nm * nm + fabsf(s[9].x) + 2.f * fabsf(s[10].x);
  }
  __device__ static float2 aentry_df64(const float2* s, int i, int J, int k, int L) {
    float2 v = df64_neg(df64_mul(s[11], df64_mul(s[i * 3 + J], s[k * 3 + L])));
    if (i == J && k == L) v = df64_add(v, s[9]);
    if (i == k && J == L) v = df64_add(v, s[10]);
    if (i == L && J == k) v = df64_add(v, s[10]);
    return v;
  }
  // C_iJkL = kap d_iJ d_kL + 2 mu th (I_sym - 1/3 d_iJ d_kL) - 2 mu thb n_iJ n_kL
  template <typename Real>
  __device__ static void aentries(const Real* scr, int i, Real* out) {
    const Real* n = scr;
    const Real kp = scr[9], mt = scr[10], mb = scr[11];
#pragma unroll
    for (int J = 0; J < 3; ++J)
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int L = 0; L < 3; ++L) {
          const Real dij = (i == J) ? Real(1) : Real(0), dkl = (k == L) ? Real(1) : Real(0);
          const Real isym = Real(0.5) * (Real((i == k) && (J == L)) + Real((i == L) && (J == k)));
          out[J * 9 + k * 3 + L] = kp * dij * dkl + mt * (isym - dij * dkl / Real(3)) - mb * n[i * 3 + J] * n[k * 3 + L];
        }
  }
};

// ---------------------------------------------------------------------------
// Mechanics (test/mechanics/TestMechanicsCommon.jl:140-190 with
// src/Formulations.jl:462-576): f = JxW G P, K = JxW G A G^T with
// G[(a,i),(i,J)] = dN_X[a][J].  Thread (r = a*3+i, cs) owns row r, column
// chunk cs:  R_r += sum_J dNX_aJ P'_iJ;  t_kL = sum_J dNX_aJ A'_iJkL;
// K_r,(b,k) += sum_L t_kL dNX_bL.
// ---------------------------------------------------------------------------
// One tile of EPB elements (thread (tx, ty): row/column chunk tx of element ty),
// shared by the kernel below and the single-launch kernel of mixed blocks.  In
// a CTA of NTHR > EPB * TPE threads the slots ty >= EPB are idle: they pass
// every barrier and touch no memory.
template <int ET, class Model, typename Real, int EPB, int CSPLIT, bool WANT_R, bool WANT_K,
          int NTHR = EPB * 3 * Elem<ET>::NNPE * CSPLIT>
__device__ __forceinline__ void mech_element_tile(const ElemArgs& g, unsigned tile, int tx, int ty,
                                                  unsigned char* smem_raw) {
  using E = Elem<ET>;
  using L = RefLayout<ET>;
  constexpr int D = 3, A = E::NNPE, NQ = E::NQ, NDOF = 3 * A, TPE = NDOF * CSPLIT;
  constexpr bool HAS_IDLE = NTHR > EPB * TPE;
  constexpr int CW = (A + CSPLIT - 1) / CSPLIT;  // nodes b per column chunk
  constexpr int NS = Model::NS, SCR = Model::SCR;
  // carve shared memory
  double* s_ref = reinterpret_cast<double*>(smem_raw);
  double* s_x_all = s_ref + ((L::SIZE + 1) & ~1);
  double* s_u_all = s_x_all + EPB * A * D;
  Real* s_dNX_all = reinterpret_cast<Real*>(s_u_all + EPB * A * D);
  Real* s_jxw_all = s_dNX_all + EPB * NQ * A * D;
  Real* s_P_all = s_jxw_all + EPB * NQ;
  Real* s_scr_all = s_P_all + EPB * NQ * 9;
  Real* s_A_all = s_scr_all + EPB * NQ * SCR;
  int* s_conn_all = reinterpret_cast<int*>(s_A_all + (WANT_K ? EPB * NQ * 81 : 0));

  // FP64: the tangent contraction runs in double-float on the FP32 pipes, from
  // (hi, lo) splits of the shape gradients and of A (written over A in place)
  constexpr bool DF = std::is_same<Real, double>::value;
  float2* s_dNXf_all = reinterpret_cast<float2*>(s_conn_all + ((EPB * A + 3) & ~3));
  // FP32-element: FP32 copy of the reference tables, FP64-differenced coordinates
  float* s_reff = reinterpret_cast<float*>(s_conn_all + ((EPB * A + 3) & ~3));
  float* s_xd_all = s_reff + ((L::SIZE + 3) & ~3);

  const int64_t e = (HAS_IDLE && ty >= EPB) ? g.ne : int64_t(tile) * EPB + ty;  // idle slot: not live
  double* s_x = s_x_all + ty * A * D;
  double* s_u = s_u_all + ty * A * D;
  Real* s_dNX = s_dNX_all + ty * NQ * A * D;
  Real* s_jxw = s_jxw_all + ty * NQ;
  Real* s_P = s_P_all + ty * NQ * 9;
  Real* s_scr = s_scr_all + ty * NQ * SCR;
  Real* s_A = s_A_all + ty * NQ * 81;
  float2* s_dNXf = s_dNXf_all + ty * NQ * A * D;
  stage_element<ET, 3, EPB, TPE, NTHR>(g, e, tx, ty, s_ref, s_conn_all + ty * A, s_x, s_u);
  const bool live = e < g.ne;
  float* s_xd = s_xd_all + ty * A * D;
  if constexpr (!DF) {
    if (!HAS_IDLE || ty < EPB)
      for (int i = ty * TPE + tx; i < L::SIZE; i += EPB * TPE) s_reff[i] = float(s_ref[i]);
    if (live)
      for (int i = tx; i < A * D; i += TPE) s_xd[i] = float(s_x[i] - s_x[i % D]);
    __syncthreads();
  }

  // quadrature-point kinematics + constitutive update, one thread per point: the
  // CTA's EPB * NQ points go to its first threads so that every warp issuing this
  // (FP64 in the FP64 variant) work has all its lanes busy
  for (int w = ty * TPE + tx; w < EPB * NQ && (!HAS_IDLE || ty < EPB); w += EPB * TPE) {
    const int el = w / NQ, q = w % NQ;
    const int64_t ee = int64_t(tile) * EPB + el;
    if (ee >= g.ne) continue;
    const double* px = s_x_all + el * A * D;
    const double* pu = s_u_all + el * A * D;
    Real* dNX = s_dNX_all + (el * NQ + q) * A * D;
    double jxw;
    if constexpr (DF)
      jxw = map_point<ET, Real>(s_ref, q, px, dNX, nullptr);
    else
      jxw = map_point_mixed<ET>(s_ref, s_reff, q, px, s_xd_all + el * A * D, dNX);
    s_jxw_all[el * NQ + q] = Real(jxw);
    Real gu[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        Real s = 0;
#pragma unroll
        for (int a = 0; a < A; ++a) s = fma(Real(pu[a * 3 + i]), dNX[a * 3 + j], s);
        gu[i][j] = s;
      }
    const double* so = NS ? g.state_old + (ee * NQ + q) * NS : nullptr;
    double* sn = (NS && g.state_new) ? g.state_new + (ee * NQ + q) * NS : nullptr;
    Real* pP = s_P_all + (el * NQ + q) * 9;
    Real* pscr = s_scr_all + (el * NQ + q) * SCR;
    if constexpr (Model::USES_CLOSURE)
      Model::point_closure(g.closure, g.props, gu, Real(jxw), so, sn, pP, pscr);
    else
      Model::point(g.props, gu, Real(jxw), so, sn, pP, pscr);
  }
  __syncthreads();
  // JxW-scaled tangent entries A'_iJkL, one (q, i) per thread
  if (WANT_K && live) {
    for (int w = tx; w < NQ * 3; w += TPE) {
      const int q = w / 3, i = w % 3;
      Real* Aq = s_A + q * 81 + i * 27;
      Model::aentries(s_scr + q * SCR, i, Aq);
      if constexpr (DF) {
        float2* Af = reinterpret_cast<float2*>(Aq);
        for (int m = 0; m < 27; ++m) Af[m] = df64_split(double(Aq[m]));
      }
    }
    if constexpr (DF) {
      for (int w = tx; w < NQ * A * D; w += TPE) s_dNXf[w] = df64_split(double(s_dNX[w]));
    }
  }
  __syncthreads();
  if (!live) return;

  const int r = tx % NDOF, cs = tx / NDOF;
  const int a = r / 3, i = r % 3;
  const int b0 = cs * CW;
  if constexpr (DF) {
    if (WANT_K) {
      float2 Kf[CW * 3];
#pragma unroll
      for (int c = 0; c < CW * 3; ++c) Kf[c] = make_float2(0.f, 0.f);
      for (int q = 0; q < NQ; ++q) {
        const float2* dNf = s_dNXf + q * A * D;
        const float2 g0 = dNf[a * 3 + 0], g1 = dNf[a * 3 + 1], g2 = dNf[a * 3 + 2];
        const float2* Ai = reinterpret_cast<const float2*>(s_A + q * 81 + i * 27);
        float2 t[9];
#pragma unroll
        for (int kl = 0; kl < 9; ++kl) t[kl] = df64_dot3(g0, Ai[kl], g1, Ai[9 + kl], g2, Ai[18 + kl]);
#pragma unroll
        for (int bb = 0; bb < CW; ++bb) {
          const int b = b0 + bb;
          if (b < A) {
            const float2 h0 = dNf[b * 3 + 0], h1 = dNf[b * 3 + 1], h2 = dNf[b * 3 + 2];
#pragma unroll
            for (int k = 0; k < 3; ++k)
              Kf[bb * 3 + k] = df64_dot3_acc(Kf[bb * 3 + k], t[k * 3 + 0], h0, t[k * 3 + 1], h1, t[k * 3 + 2], h2);
          }
        }
      }
      float2* Ke = static_cast<float2*>(g.Ke) + (e * NDOF + r) * NDOF + b0 * 3;
#pragma unroll
      for (int c = 0; c < CW * 3; ++c)
        if (b0 * 3 + c < NDOF) Ke[c] = Kf[c];
    }
    if (WANT_R && cs == 0) {
      double R = 0;
      for (int q = 0; q < NQ; ++q) {
        const double* dNX = s_dNX + q * A * D;
        const double* P = s_P + q * 9 + i * 3;
        R = fma(dNX[a * 3], P[0], fma(dNX[a * 3 + 1], P[1], fma(dNX[a * 3 + 2], P[2], R)));
      }
      static_cast<double*>(g.Re)[e * NDOF + r] = R;
    }
  } else {
  Real Krow[CW * 3];
#pragma unroll
  for (int c = 0; c < CW * 3; ++c) Krow[c] = 0;
  Real R = 0;
  for (int q = 0; q < NQ; ++q) {
    const Real* dNX = s_dNX + q * A * D;
    const Real g0 = dNX[a * 3 + 0], g1 = dNX[a * 3 + 1], g2 = dNX[a * 3 + 2];
    if (WANT_R && cs == 0) {
      const Real* P = s_P + q * 9 + i * 3;
      R = fma(g0, P[0], fma(g1, P[1], fma(g2, P[2], R)));
    }
    if (WANT_K) {
      const Real* Ai = s_A + q * 81 + i * 27;
      Real t[9];
#pragma unroll
      for (int kl = 0; kl < 9; ++kl) t[kl] = fma(g0, Ai[kl], fma(g1, Ai[9 + kl], g2 * Ai[18 + kl]));
#pragma unroll
      for (int bb = 0; bb < CW; ++bb) {
        const int b = b0 + bb;
        if (b < A) {
          const Real h0 = dNX[b * 3 + 0], h1 = dNX[b * 3 + 1], h2 = dNX[b * 3 + 2];
#pragma unroll
          for (int k = 0; k < 3; ++k)
            Krow[bb * 3 + k] += fma(t[k * 3 + 0], h0, fma(t[k * 3 + 1], h1, t[k * 3 + 2] * h2));
        }
      }
    }
  }
  if (WANT_K) {
    typename WS<Real>::T* Ke = static_cast<typename WS<Real>::T*>(g.Ke) + (e * NDOF + r) * NDOF + b0 * 3;
#pragma unroll
    for (int c = 0; c < CW * 3; ++c)
      if (b0 * 3 + c < NDOF) Ke[c] = WS<Real>::from(Krow[c]);
  }
  if (WANT_R && cs == 0) static_cast<Real*>(g.Re)[e * NDOF + r] = R;
  }
}

template <int ET, class Model, typename Real, int EPB, int CSPLIT, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(EPB * 3 * Elem<ET>::NNPE * CSPLIT)
    mech_element_kernel(ElemArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  mech_element_tile<ET, Model, Real, EPB, CSPLIT, WANT_R, WANT_K>(g, blockIdx.x, threadIdx.x, threadIdx.y, smem_raw);
}

template <int ET, class Model, typename Real, int EPB, bool WANT_K>
constexpr size_t mech_smem_bytes() {
  using E = Elem<ET>;
  constexpr int A = E::NNPE, NQ = E::NQ;
  constexpr bool DF = std::is_same<Real, double>::value;
  return sizeof(double) * (((RefLayout<ET>::SIZE + 1) & ~1) + 2 * EPB * A * 3) +
         sizeof(Real) * (EPB * NQ * A * 3 + EPB * NQ + EPB * NQ * 9 + EPB * NQ * Model::SCR +
                         (WANT_K ? EPB * NQ * 81 : 0)) +
         sizeof(int) * ((EPB * A + 3) & ~3) + (DF && WANT_K ? sizeof(float2) * EPB * NQ * A * 3 : 0) +
         (DF ? 0 : sizeof(float) * (((RefLayout<ET>::SIZE + 3) & ~3) + EPB * A * 3)) + 16;
}

// ---------------------------------------------------------------------------
// Node gather: deterministic element-ordered reduction into CSC nzval and the
// residual over unknowns.
// ---------------------------------------------------------------------------
struct BlockInfo {
  int64_t elem_start;   // first global element id of the block
  int64_t ke_off;       // Ke offset (entries) of the block
  int64_t re_off;       // Re offset (entries) of the block
  int64_t conn_off;     // offset into conn (entries)
  int64_t epos_off;     // offset into epos (entries)
  int nnpe;
  int ndof;
  int layout;           // element-matrix layout, see ke_index
};

constexpr int MAX_BLOCKS = 16;

// Element-matrix workspace layouts.  Entry (row (a,k), column (b,i)) of one
// element, NF fields, A nodes:
//   KE_ROW_MAJOR:   (a*NF + k)*NF*A + b*NF + i        (K_e row-major)
//   KE_NODE_ROWS:   ((a*NF + k)*NF + i)*A + b         (column node fastest; used by
//                   the hex8 mechanics kernels so that the gather reads, per row
//                   component and column component, the 8 column nodes as two
//                   16-byte vectors)
//   KE_PAIRS:       the symmetric half only (NF = 3): node pair (x, y), x <= y,
//                   p = x*(2A - x + 1)/2 + y - x, holds K_(x,k'),(y,i') at
//                   p*9 + 3k' + i'; an entry with a > b is read from pair (b, a)
//                   transposed (K = K^T).  A(A+1)/2 * 9 entries per element; written
//                   by the class tensor-core kernel (fec_class_tc.cu)
enum { KE_ROW_MAJOR = 0, KE_NODE_ROWS = 1, KE_PAIRS = 2 };

// Offset of entry (row (a,k), column (b,i)) of one element in the KE_PAIRS layout.
__host__ __device__ __forceinline__ int pair_entry(int A, int a, int k, int b, int i) {
  const bool own = a <= b;
  const int x = own ? a : b, y = own ? b : a;
  return (x * (2 * A - x + 1) / 2 + (y - x)) * 9 + (own ? k * 3 + i : i * 3 + k);
}

struct GatherArgs {
  int64_t nn;                  // nodes
  int nf;                      // fields per node
  int nblocks;
  BlockInfo blk[MAX_BLOCKS];
  const int64_t* nadj_ptr;     // [nn+1]
  const uint32_t* nadj;        // global element * 32 + local node (fewer than 2^27 elements)
  const int32_t* conn;         // all blocks, 0-based
  const uint16_t* epos;        // [elem][a][b] row offset of node conn[b] inside node conn[a]'s columns
  const uint8_t* umask;        // per node: bit f set when dof (node, f) is unknown
  const int64_t* col_base;     // per node: nzval offset of its first column
  const int32_t* col_len;      // per node: rows per column
  const int64_t* dof_to_unknown;  // per dof: 0-based unknown index or -1
  const void* Ke;
  const void* Re;
  double* nzval;               // may be null
  double* R_u;                 // may be null
  int acc_stride;              // doubles of accumulator per warp
  const int32_t* nodes;        // node_gather_kernel: gather nodes[0 .. nnodes) instead of 0 .. nn (may be null)
  int64_t nnodes;
};

// Bit 7 of umask[n]: node n and every node it couples to have all NF components
// unknown, so CSC positions need no per-neighbour lookups.
constexpr unsigned UMASK_FULL_NBR = 0x80u;

// Exact float -> double widening with integer operations only (the hardware
// conversion issues on the FP64 pipe, 1/64 of the FP32 rate on this part).
// Handles zero, subnormal, inf and nan without branches.
__device__ __forceinline__ double widen_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint64_t sign = uint64_t(u & 0x80000000u) << 32;
  const uint32_t ex = (u >> 23) & 0xffu;
  const uint32_t m = u & 0x7fffffu;
  // normal: rebias the exponent
  uint64_t bits = sign | (uint64_t(ex + (1023u - 127u)) << 52) | (uint64_t(m) << 29);
  // subnormal: normalise the mantissa (m != 0, ex == 0)
  const int lz = __clz(m) - 8;  // leading zeros inside the 23-bit field, plus one
  const uint64_t sub = sign | (uint64_t(1023 - 126 - lz) << 52) | (uint64_t((m << lz) & 0x7fffffu) << 29);
  bits = (ex == 0u) ? (m == 0u ? sign : sub) : bits;
  bits = (ex == 0xffu) ? (sign | (uint64_t(0x7ffu) << 52) | (uint64_t(m) << 29)) : bits;
  return __longlong_as_double(int64_t(bits));
}

// Float -> double widening for normal floats and zeros in six integer
// operations (the exponent rebias is one add on the high word); subnormals,
// inf and nan go through widen_exact.
__device__ __forceinline__ double widen(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t mag = u & 0x7FFFFFFFu;
  if (mag - 0x00800000u >= 0x7F000000u && mag != 0u) return widen_exact(f);
  const uint32_t hiw = (u & 0x80000000u) | (mag == 0u ? 0u : (mag >> 3) + (896u << 20));
  return __hiloint2double(int(hiw), int(u << 29));
}

// A residual contribution as a double: doubles as they are, floats widened
// exactly on the integer pipes (a conversion would issue on the FP64 pipe).
__device__ __forceinline__ double to_double(double x) { return x; }
__device__ __forceinline__ double to_double(float x) { return widen(x); }

// Accumulator of the node gather: a compensated FP32 pair (hi, lo).  Adding a
// float recovers its rounding error exactly with TwoSum (Knuth); adding a
// double-float pair is a df64 addition.  Either keeps the sum to about 2^-48
// relative -- FP64-class accumulation carried by the FP32 pipes -- and only the
// final hi + lo is formed in FP64.
struct GatherAcc {
  static constexpr int WORDS = 2;  // 4-byte words per entry
  __device__ static void zero(float* base, int j) { reinterpret_cast<float2*>(base)[j] = make_float2(0.f, 0.f); }
  __device__ static float2 plus(float2 a, float v) {
    const float s = __fadd_rn(a.x, v);
    const float bp = __fsub_rn(s, a.x);
    const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bp)), __fsub_rn(v, bp));
    return make_float2(s, __fadd_rn(a.y, err));
  }
  __device__ static float2 plus(float2 a, float2 v) { return df64_add(a, v); }
  template <typename W>
  __device__ static void add(float* base, int j, W v) {
    float2* p = reinterpret_cast<float2*>(base) + j;
    *p = plus(*p, v);
  }
  __device__ static double value(float2 a) { return widen(a.x) + widen(a.y); }
  __device__ static double value(const float* base, int j) { return value(reinterpret_cast<const float2*>(base)[j]); }
};

// Adds the contributions of adjacency entries [p, pend) -- all from one element
// block with A nodes per element -- to the node's accumulator, in entry
// (= increasing element) order.  Each lane fetches one adjacency entry, the
// entries are broadcast by shuffles, and the row loads of up to CH elements
// are all issued before their additions, so a warp keeps CH*VPL loads in
// flight per lane instead of a dependent load chain per element.
template <typename Real, int NF, int A, int BUDGET>
__device__ __forceinline__ void gather_run(const GatherArgs& g, const BlockInfo& B, int64_t p, int64_t pend, unsigned um,
                                           bool fast, int Ln, float* acc, double& racc, int lane, bool wantK,
                                           bool wantR) {
  constexpr int NDOF = NF * A;
  constexpr int TOTAL = NF * NDOF;                         // values of one element's rows for this node
  constexpr int VPL = (TOTAL + 31) / 32;                   // values per lane per element
  constexpr int CH = VPL >= BUDGET ? 1 : (BUDGET / VPL > 8 ? 8 : BUDGET / VPL);
  using RT = typename RE<Real>::T;
  const Real* Ke = static_cast<const Real*>(g.Ke) + B.ke_off;
  const RT* Re = static_cast<const RT*>(g.Re) + B.re_off;
  const bool pairs = B.layout == KE_PAIRS;
  constexpr int NPW = A * (A + 1) / 2 * 9;  // KE_PAIRS entries per element
  for (; p < pend; p += 32) {
    const int64_t left32 = pend - p;
    const int n32 = left32 < 32 ? int(left32) : 32;
    const uint32_t mine = lane < n32 ? g.nadj[p + lane] : 0u;
    for (int c0 = 0; c0 < n32; c0 += CH) {
      const int nh = (n32 - c0) < CH ? (n32 - c0) : CH;
      Real v[CH][VPL];
      int pos[CH][VPL];
      RT rv[CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const uint32_t packed = __shfl_sync(0xffffffffu, mine, (c0 + c) & 31);
        rv[c] = RT(0);
#pragma unroll
        for (int j = 0; j < VPL; ++j) pos[c][j] = -1;
        if (c < nh) {
          const int le = int(packed >> 5) - int(B.elem_start);
          const int a = int(packed & 31u);
          const uint64_t row0 = uint64_t(uint32_t(le)) * NDOF + uint32_t(a * NF);  // first row of node a
          if (wantR) rv[c] = Re[row0 + lane];
          if (wantK) {
            const Real* Krows = Ke + row0 * NDOF;
            const Real* Kel = Ke + uint64_t(uint32_t(le)) * NPW;
            const uint16_t* ep = g.epos + B.epos_off + (uint64_t(uint32_t(le)) * A + a) * A;
#pragma unroll
            for (int j = 0; j < VPL; ++j) {
              const int t = lane + 32 * j;
              if (t < TOTAL) {
                const int k = t / NDOF, rem = t % NDOF;
                const int b = rem / NF, i = rem % NF;
                v[c][j] = pairs ? Kel[pair_entry(A, a, k, b, i)] : Krows[t];
                if (fast) {
                  pos[c][j] = k * Ln + ep[b] + i;
                } else if ((um >> k) & 1u) {
                  const unsigned umm = g.umask[g.conn[B.conn_off + int64_t(le) * A + b]] & ~UMASK_FULL_NBR;
                  if ((umm >> i) & 1u)
                    pos[c][j] = __popc(um & ((1u << k) - 1u)) * Ln + ep[b] + __popc(umm & ((1u << i) - 1u));
                }
              }
            }
          }
        }
      }
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        if (c < nh) {
          racc += to_double(rv[c]);
          if (wantK) {
            // one element's values of this lane go to distinct positions: loads,
            // additions and stores are batched
            float2* A2 = reinterpret_cast<float2*>(acc);
            float2 sv[VPL];
#pragma unroll
            for (int j = 0; j < VPL; ++j)
              if (pos[c][j] >= 0) sv[j] = A2[pos[c][j]];
#pragma unroll
            for (int j = 0; j < VPL; ++j)
              if (pos[c][j] >= 0) A2[pos[c][j]] = GatherAcc::plus(sv[j], v[c][j]);
            __syncwarp();
          }
        }
      }
    }
  }
}

// Same for a run whose element size is only known at run time (meshes whose
// blocks have different element sizes).
template <typename Real, int NF>
__device__ __forceinline__ void gather_run_generic(const GatherArgs& g, const BlockInfo& B, int64_t p, int64_t pend,
                                                   unsigned um, bool fast, int Ln, float* acc, double& racc, int lane,
                                                   bool wantK, bool wantR) {
  using RT = typename RE<Real>::T;
  const int A = B.nnpe, NDOF = B.ndof;
  const bool node_rows = B.layout == KE_NODE_ROWS, pairs = B.layout == KE_PAIRS;
  const int64_t npw = int64_t(A) * (A + 1) / 2 * 9;  // KE_PAIRS entries per element
  const Real* Ke = static_cast<const Real*>(g.Ke) + B.ke_off;
  const RT* Re = static_cast<const RT*>(g.Re) + B.re_off;
  for (; p < pend; ++p) {
    const uint32_t packed = g.nadj[p];
    const int64_t le = int64_t(packed >> 5) - B.elem_start;
    const int a = int(packed & 31u);
    if (wantR) racc += to_double(Re[le * NDOF + a * NF + lane]);
    if (wantK) {
      const Real* Krows = Ke + (le * NDOF + int64_t(a) * NF) * NDOF;
      const Real* Kel = Ke + le * npw;
      const uint16_t* ep = g.epos + B.epos_off + (le * A + a) * A;
      const int32_t* cn = g.conn + B.conn_off + le * A;
#pragma unroll
      for (int k = 0; k < NF; ++k) {
        if (!((um >> k) & 1u)) continue;
        const int kb = __popc(um & ((1u << k) - 1u)) * Ln;
        // lanes over the element's columns (b, i) of row component k
        for (int rem = lane; rem < NDOF; rem += 32) {
          const int b = rem / NF, i = rem - b * NF;
          int pos;
          if (fast) {  // every neighbour component is unknown: no mask lookups
            pos = kb + ep[b] + i;
          } else {
            const unsigned umm = g.umask[cn[b]] & ~UMASK_FULL_NBR;
            if (!((umm >> i) & 1u)) continue;
            pos = kb + ep[b] + __popc(umm & ((1u << i) - 1u));
          }
          GatherAcc::add(acc, pos,
                         pairs ? Kel[pair_entry(A, a, k, b, i)] : Krows[node_rows ? (k * NF + i) * A + b : k * NDOF + rem]);
        }
      }
      __syncwarp();
    }
  }
}

// four double-float workspace entries (one 32-byte vector)
struct alignas(32) F2x4 {
  float2 x, y, z, w;
};

// Vector hex8 in the KE_NODE_ROWS layout, for nodes whose whole neighbourhood
// is unknown: lane l < 18 owns (row component k, column component i) = (l/2)
// and the column nodes b = 4(l%2) .. 4(l%2)+3, read as one 16-byte (FP32) or
// two 16-byte (FP64) vectors, with their CSC row offsets from one 8-byte load
// of the element map.  Positions are k*Ln + i + epos[b]: two integer ops per
// value.
template <typename Real>
__device__ __forceinline__ void gather_run_hex8v(const GatherArgs& g, const BlockInfo& B, int64_t p, int64_t pend,
                                                 int Ln, float* acc, double& racc, int lane, bool wantK, bool wantR) {
  constexpr int CH = sizeof(Real) == 8 ? 4 : 6;
  using V4 = typename std::conditional<sizeof(Real) == 4, float4, F2x4>::type;
  using RT = typename RE<Real>::T;
  const Real* Ke = static_cast<const Real*>(g.Ke) + B.ke_off;
  const RT* Re = static_cast<const RT*>(g.Re) + B.re_off;
  const bool kl = lane < 18;
  const int ki = lane >> 1, bh = lane & 1;
  const int base = (ki / 3) * Ln + (ki % 3);
  for (; p < pend; p += 32) {
    const int64_t left32 = pend - p;
    const int n32 = left32 < 32 ? int(left32) : 32;
    const uint32_t mine = lane < n32 ? g.nadj[p + lane] : 0u;
    for (int c0 = 0; c0 < n32; c0 += CH) {
      const int nh = (n32 - c0) < CH ? (n32 - c0) : CH;
      V4 v[CH];
      uint2 ep[CH];
      RT rv[CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const uint32_t packed = __shfl_sync(0xffffffffu, mine, (c0 + c) & 31);
        rv[c] = RT(0);
        if (c < nh) {
          const uint32_t le = (packed >> 5) - uint32_t(B.elem_start);
          const uint32_t a = packed & 31u;
          // 32-bit offsets: element rows (le*576 < 2^32 for < 2^22 elements per block is not
          // assumed; the 576-entry row block index is widened once)
          if (wantR) rv[c] = Re[uint64_t(le * 24u + a * 3u) + lane];
          if (wantK && kl) {
            v[c] = *reinterpret_cast<const V4*>(Ke + uint64_t(le) * 576u + (a * 72u + ki * 8u + bh * 4u));
            ep[c] = *reinterpret_cast<const uint2*>(g.epos + B.epos_off + uint64_t(le) * 64u + (a * 8u + bh * 4u));
          }
        }
      }
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        if (c < nh) {
          racc += to_double(rv[c]);
          if (wantK) {
            if (kl) {
              // the four columns of one element go to four distinct positions, so
              // their read-modify-writes are issued as one batch of loads, four
              // independent additions and one batch of stores
              float2* A2 = reinterpret_cast<float2*>(acc);
              const int p0 = base + int(ep[c].x & 0xffffu), p1 = base + int(ep[c].x >> 16);
              const int p2 = base + int(ep[c].y & 0xffffu), p3 = base + int(ep[c].y >> 16);
              float2 s0 = A2[p0], s1 = A2[p1], s2 = A2[p2], s3 = A2[p3];
              s0 = GatherAcc::plus(s0, v[c].x);
              s1 = GatherAcc::plus(s1, v[c].y);
              s2 = GatherAcc::plus(s2, v[c].z);
              s3 = GatherAcc::plus(s3, v[c].w);
              A2[p0] = s0;
              A2[p1] = s1;
              A2[p2] = s2;
              A2[p3] = s3;
            }
            __syncwarp();
          }
        }
      }
    }
  }
}

// One warp per node.  A > 0: every block has A nodes per element; A == 0: mixed.
template <typename Real, int NF, int A, int WPB, int MINB, int BUDGET>
__global__ void __launch_bounds__(WPB * 32, MINB) node_gather_kernel(GatherArgs g) {
  extern __shared__ __align__(16) float s_acc[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int64_t n = int64_t(blockIdx.x) * WPB + warp;
  if (g.nodes) {
    if (n >= g.nnodes) return;
    n = g.nodes[n];
  } else if (n >= g.nn) {
    return;
  }
  // the node's own entries, all issued before any is used (one memory latency)
  const unsigned um_raw = g.umask[n];
  const int Ln = g.col_len[n];
  int64_t p = g.nadj_ptr[n];
  const int64_t p1 = g.nadj_ptr[n + 1];
  const int64_t col0 = g.nzval ? g.col_base[n] : 0;
  const int64_t dtu = (g.R_u && lane < NF) ? g.dof_to_unknown[n * NF + lane] : 0;
  const bool fast = (um_raw & UMASK_FULL_NBR) != 0;
  const unsigned um = um_raw & ~UMASK_FULL_NBR;
  if (um == 0) return;
  const int ncols = __popc(um);
  float* acc = s_acc + warp * g.acc_stride * GatherAcc::WORDS;
  const bool wantK = g.nzval != nullptr;
  const bool wantR = g.R_u != nullptr && lane < NF && ((um >> lane) & 1u);
  if (wantK)
    for (int j = lane; j < ncols * Ln; j += 32) GatherAcc::zero(acc, j);
  double racc = 0.0;  // the residual is summed in FP64, in increasing element order
  __syncwarp();
  while (p < p1) {
    // the run of entries from one element block
    const int64_t ge = int64_t(g.nadj[p] >> 5);
    int bi = 0;
    while (bi + 1 < g.nblocks && ge >= g.blk[bi + 1].elem_start) ++bi;
    const BlockInfo& B = g.blk[bi];
    int64_t q = p1;
    if (bi + 1 < g.nblocks) {
      const int64_t bend = g.blk[bi + 1].elem_start;
      q = p + 1;
      while (q < p1 && int64_t(g.nadj[q] >> 5) < bend) ++q;
    }
    if constexpr (A == 8 && NF == 3) {
      if (fast && B.layout == KE_NODE_ROWS)
        gather_run_hex8v<Real>(g, B, p, q, Ln, acc, racc, lane, wantK, wantR);
      else
        gather_run_generic<Real, NF>(g, B, p, q, um, fast, Ln, acc, racc, lane, wantK, wantR);
    } else if constexpr (A > 0) {
      gather_run<Real, NF, A, BUDGET>(g, B, p, q, um, fast, Ln, acc, racc, lane, wantK, wantR);
    } else {
      gather_run_generic<Real, NF>(g, B, p, q, um, fast, Ln, acc, racc, lane, wantK, wantR);
    }
    p = q;
  }
  if (wantK) {
    double* out = g.nzval + col0;
    for (int j = lane; j < ncols * Ln; j += 32) out[j] = GatherAcc::value(acc, j);
  }
  if (wantR) g.R_u[dtu] = racc;
}

// ---------------------------------------------------------------------------
// Software-pipelined node gather for meshes of one hex8 mechanics block (the
// KE_NODE_ROWS layout, or KE_PAIRS: the FP64 tensor-core kernel's symmetric half).  Each warp walks the nodes gw, gw + GW, ... (GW =
// warps in the grid).  While it accumulates node i from shared memory, the
// rows its elements hold for node i+1 (8 x 72 entries), their element-map
// entries and residual values are already on their way into the warp's other
// stage buffer by cp.async, and node i+2's adjacency entries are in
// registers, so the three dependent loads of a node (adjacency, element rows,
// accumulate) no longer serialise per node.  The accumulation is the one of
// gather_run_hex8v, value for value and in the same element order, so the
// results are bitwise those of node_gather_kernel.  Nodes outside the fast
// path (a Dirichlet dof in the neighbourhood, or more than 8 adjacent
// elements) are gathered in place by the general routine.
// ---------------------------------------------------------------------------
namespace gp {
constexpr int WPB = 8;
constexpr int MAXE = 8;  // elements staged per node
// PAIRS (the KE_PAIRS layout, 8-byte entries): node a's eight 9-entry pair blocks of
// an element, each copied as the 80 bytes from the 16-byte boundary at or below its
// start (a block of pair p starts 8 bytes past that boundary when p is odd)
template <typename Real, bool PAIRS = false>
struct Stage {
  static constexpr int BLK = 80;                                 // staged bytes per pair block
  static constexpr int K_BYTES = PAIRS ? MAXE * 8 * BLK : MAXE * 72 * int(sizeof(Real));  // node a's 72 entries
  static constexpr int EP_OFF = K_BYTES;                         // uint16 [MAXE][8] element-map entries
  static constexpr int R_OFF = EP_OFF + MAXE * 16;               // RE<Real> [MAXE][3] residual values
  static constexpr int BYTES = (R_OFF + MAXE * 3 * int(sizeof(typename RE<Real>::T)) + 15) / 16 * 16;
  static constexpr int CHUNKS = PAIRS ? 8 * BLK / 16 : 72 * int(sizeof(Real)) / 16;  // 16-byte copies per element
};
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
template <int BYTES>
__device__ __forceinline__ void cp_small(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

struct NodeMeta {
  int64_t n;        // node, or -1 past the end
  int64_t p0, p1;   // adjacency entries [p0, p1)
  unsigned um;      // umask with the full-neighbourhood bit
  int Ln;           // rows per column
  int cnt;          // adjacency entries                             (stage b)
  uint32_t adj;     // this lane's adjacency entry (lane < cnt)      (stage b)
  bool pipe;        // staged through shared memory                  (stage b)
  int64_t col0;     // first nzval entry of the node's columns       (stage c)
  int64_t dtu;      // lanes 0-2: unknown of the node's component    (stage c)
};

// The node's metadata in three stages, each a node apart, so that no global load
// is used in the iteration that issues it: (a) the node's own entries, (b) its
// adjacency entries, addressed by (a), (c) where its columns and residual go.
__device__ __forceinline__ NodeMeta meta_a(const GatherArgs& g, int64_t n) {
  NodeMeta m;
  m.n = n < g.nn ? n : -1;
  m.p0 = m.p1 = 0;
  m.um = 0;
  m.Ln = 0;
  m.cnt = 0;
  m.adj = 0;
  m.pipe = false;
  m.col0 = m.dtu = 0;
  if (m.n < 0) return m;
  m.um = g.umask[n];
  m.Ln = g.col_len[n];
  m.p0 = g.nadj_ptr[n];
  m.p1 = g.nadj_ptr[n + 1];
  return m;
}
__device__ __forceinline__ void meta_b(const GatherArgs& g, NodeMeta& m, int lane) {
  if (m.n < 0) return;
  m.cnt = int(m.p1 - m.p0);
  m.pipe = (m.um & UMASK_FULL_NBR) != 0 && m.cnt >= 1 && m.cnt <= MAXE;
  if (m.pipe && lane < m.cnt) m.adj = g.nadj[m.p0 + lane];
}
__device__ __forceinline__ void meta_c(const GatherArgs& g, NodeMeta& m, int lane) {
  if (m.n < 0) return;
  if (g.nzval) m.col0 = g.col_base[m.n];
  if (g.R_u && lane < 3) m.dtu = g.dof_to_unknown[m.n * 3 + lane];
}

// pair index of the node pair (x, y), x <= y, of a hex8 element
__device__ __forceinline__ int hex8_pair(int x, int y) { return (x * (15 - x)) / 2 + y; }

// Offsets of the KE_PAIRS staging (shared memory, built once per CTA):
//   chunk[a][w]: byte offset in an element's 2,592 pair bytes of 16-byte chunk w
//     (part w % 5 of the block of column node w / 5) of node a's rows; the 80-byte
//     window stays inside the element's entries
//   blk[a][b]:   byte offset in the staged 640 bytes of node a's block for column
//     node b, bit 15 set when the block is pair (a, b) itself (a <= b: entry 3k + i
//     holds K_(a,k),(b,i)), clear for pair (b, a) (entry 3i + k)
struct PairTables {
  uint16_t chunk[8][40];
  uint16_t blk[8][8];
};
__device__ __forceinline__ void build_pair_tables(PairTables& t) {
  for (int i = threadIdx.x; i < 8 * 40 + 64; i += blockDim.x) {
    if (i < 320) {
      const int a = i / 40, w = i % 40, bb = w / 5, part = w % 5;
      const int p = hex8_pair(a < bb ? a : bb, a < bb ? bb : a);
      t.chunk[a][w] = uint16_t(((p * 72) & ~15) + part * 16);
    } else {
      const int a = (i - 320) / 8, b = (i - 320) % 8;
      const int p = hex8_pair(a < b ? a : b, a < b ? b : a);
      t.blk[a][b] = uint16_t(b * 80 + (p & 1) * 8) | (a <= b ? 0x8000u : 0u);
    }
  }
}

// cp.async of node m's staged data into `st` (all 32 lanes; a commit group always
// follows).  Lane (c, sub) = (lane / 4, lane % 4) copies element c's chunks sub,
// sub + 4, ... (one shuffle per node for the element's entry).
template <typename Real, bool PAIRS>
__device__ __forceinline__ void issue(const GatherArgs& g, const NodeMeta& m, unsigned char* st, int lane,
                                      const PairTables* pt) {
  using S = Stage<Real, PAIRS>;
  using RT = typename RE<Real>::T;
  if (!m.pipe) return;
  const BlockInfo& B = g.blk[0];
  const unsigned char* Ke = reinterpret_cast<const unsigned char*>(static_cast<const Real*>(g.Ke) + B.ke_off);
  const uint16_t* ep = g.epos + B.epos_off;
  const RT* Re = static_cast<const RT*>(g.Re) + B.re_off;
  {
    const int c = lane >> 2, sub = lane & 3;
    const uint32_t packed = __shfl_sync(0xffffffffu, m.adj, c);
    if (c < m.cnt) {
      const uint64_t le = (packed >> 5) - uint32_t(B.elem_start);
      const int a = int(packed & 31u);
      if constexpr (PAIRS) {
        const unsigned char* src = Ke + le * (324u * sizeof(Real));
        unsigned char* dst = st + c * (8 * S::BLK);
        const uint16_t* ch = pt->chunk[a];
#pragma unroll
        for (int j = 0; j < S::CHUNKS / 4; ++j) cp16(dst + (sub + 4 * j) * 16, src + ch[sub + 4 * j]);
      } else {
        const unsigned char* src = Ke + (le * 576u + uint64_t(a) * 72u) * sizeof(Real);
        unsigned char* dst = st + c * (72 * sizeof(Real));
#pragma unroll
        for (int j = 0; j < (S::CHUNKS + 3) / 4; ++j)
          if (sub + 4 * j < S::CHUNKS) cp16(dst + (sub + 4 * j) * 16, src + (sub + 4 * j) * 16);
      }
    }
  }
  if (lane < m.cnt) {  // element-map row of node a: 8 uint16, 16-byte aligned
    const uint64_t le = (m.adj >> 5) - uint32_t(B.elem_start), a = m.adj & 31u;
    cp16(st + S::EP_OFF + lane * 16, ep + le * 64u + a * 8u);
  }
  {  // residual values: lane t = 3 c + i < 3 cnt (at most 24)
    const int c = lane / 3 < MAXE ? lane / 3 : MAXE - 1, i = lane - 3 * c;
    const uint32_t packed = __shfl_sync(0xffffffffu, m.adj, c);
    const uint64_t le = (packed >> 5) - uint32_t(B.elem_start), a = packed & 31u;
    if (g.R_u && lane < 3 * m.cnt)
      cp_small<sizeof(RT)>(st + S::R_OFF + lane * sizeof(RT), Re + le * 24u + a * 3u + i);
  }
}
}  // namespace gp

template <typename Real, int MINB, bool PAIRS = false>
__global__ void __launch_bounds__(gp::WPB * 32, MINB) node_gather_hex8_pipe_kernel(GatherArgs g) {
  using namespace gp;
  using S = Stage<Real, PAIRS>;
  using RT = typename RE<Real>::T;
  extern __shared__ __align__(16) unsigned char smem_g[];
  __shared__ PairTables s_pt;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if constexpr (PAIRS) {
    build_pair_tables(s_pt);
    __syncthreads();
  }
  const size_t acc_bytes = (size_t(g.acc_stride) * GatherAcc::WORDS * sizeof(float) + 15) / 16 * 16;
  unsigned char* wbase = smem_g + warp * (acc_bytes + 2 * S::BYTES);
  float* acc = reinterpret_cast<float*>(wbase);
  unsigned char* stage[2] = {wbase + acc_bytes, wbase + acc_bytes + S::BYTES};
  const int64_t GW = int64_t(gridDim.x) * WPB;
  const bool wantK = g.nzval != nullptr;
  const BlockInfo& B = g.blk[0];
  // lane (k, b) < 24 adds column node b's three entries of row component k
  const bool kl = lane < 24;
  const int lk = lane >> 3, lb = lane & 7;

  // node i is gathered while node i+1's copies are in flight, node i+2's
  // adjacency entries and node i+3's own entries are loaded
  auto next = [&](const NodeMeta& m) { return m.n < 0 ? g.nn : m.n + GW; };
  NodeMeta cur = meta_a(g, int64_t(blockIdx.x) * WPB + warp);
  meta_b(g, cur, lane);
  meta_c(g, cur, lane);
  issue<Real, PAIRS>(g, cur, stage[0], lane, &s_pt);
  commit();
  NodeMeta nxt = meta_a(g, next(cur));
  meta_b(g, nxt, lane);
  NodeMeta n2 = meta_a(g, next(nxt));
  for (int it = 0; cur.n >= 0; ++it) {
    const int s = it & 1;
    issue<Real, PAIRS>(g, nxt, stage[s ^ 1], lane, &s_pt);  // node i+1 into the other stage
    commit();
    meta_c(g, nxt, lane);
    meta_b(g, n2, lane);
    const NodeMeta n3 = meta_a(g, next(n2));
    wait_prev();                              // node i's copies (this lane's) have landed
    __syncwarp();                             // ... and every lane's
    const unsigned um = cur.um & ~UMASK_FULL_NBR;
    if (um != 0) {
      const int Ln = cur.Ln, ncols = __popc(um);
      const bool wantR = g.R_u != nullptr && lane < 3 && ((um >> lane) & 1u);
      if (wantK)
        for (int j = lane; j < ncols * Ln; j += 32) GatherAcc::zero(acc, j);
      double racc = 0.0;
      __syncwarp();
      if (cur.pipe) {
        const unsigned char* st = stage[s];
        const int base = lk * Ln;
        for (int c = 0; c < cur.cnt; ++c) {
          if (wantR) racc += to_double(reinterpret_cast<const RT*>(st + S::R_OFF)[c * 3 + lane]);
          if (wantK) {
            int a = 0;
            if constexpr (PAIRS) a = int(__shfl_sync(0xffffffffu, cur.adj, c) & 31u);
            if (kl) {
              // entries ((k*3 + i)*8 + b) of the element's rows for this node, i = 0..2, go to
              // the three adjacent positions k*Ln + epos[b] + i
              Real v0, v1, v2;
              if constexpr (PAIRS) {  // K_(a,k),(b,i): pair (a, b) entry 3k + i, or pair (b, a) entry 3i + k
                const unsigned bo = s_pt.blk[a][lb];
                const Real* blk = reinterpret_cast<const Real*>(st + c * (8 * S::BLK) + (bo & 0x7fffu));
                const bool own = (bo & 0x8000u) != 0;
                const int o = own ? lk * 3 : lk, d = own ? 1 : 3;
                v0 = blk[o];
                v1 = blk[o + d];
                v2 = blk[o + 2 * d];
              } else {
                const Real* row = reinterpret_cast<const Real*>(st) + c * 72 + lk * 24 + lb;
                v0 = row[0];
                v1 = row[8];
                v2 = row[16];
              }
              const int p = base + int(reinterpret_cast<const uint16_t*>(st + S::EP_OFF + c * 16)[lb]);
              float2* A2 = reinterpret_cast<float2*>(acc) + p;
              float2 s0 = A2[0], s1 = A2[1], s2 = A2[2];
              s0 = GatherAcc::plus(s0, v0);
              s1 = GatherAcc::plus(s1, v1);
              s2 = GatherAcc::plus(s2, v2);
              A2[0] = s0;
              A2[1] = s1;
              A2[2] = s2;
            }
            __syncwarp();
          }
        }
      } else {
        const bool fast = (cur.um & UMASK_FULL_NBR) != 0;
        const int64_t p1 = cur.p0 + cur.cnt;
        if (fast && !PAIRS)
          gather_run_hex8v<Real>(g, B, cur.p0, p1, Ln, acc, racc, lane, wantK, wantR);
        else
          gather_run_generic<Real, 3>(g, B, cur.p0, p1, um, fast, Ln, acc, racc, lane, wantK, wantR);
      }
      __syncwarp();
      if (wantK) {
        double* out = g.nzval + cur.col0;
        for (int j = lane; j < ncols * Ln; j += 32) out[j] = GatherAcc::value(acc, j);
      }
      if (wantR) g.R_u[cur.dtu] = racc;
      __syncwarp();
    }
    cur = nxt;
    nxt = n2;
    n2 = n3;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
}

}  // namespace fec
