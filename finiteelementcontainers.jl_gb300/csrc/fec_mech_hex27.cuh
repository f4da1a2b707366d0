// fec_mech_hex27.cuh -- the FP64 hex27 mechanics element (27 nodes, 27
// points): kinematics and the constitutive update in native FP64, the
// symmetric tangent contraction in double-float on the FP32 pipes.
//
// 162 contracting threads per element: thread (r, cs) owns element row r =
// (a, i) and the node blocks b = a + d (mod 27) for d in [7 cs, 7 cs + 7): with
// 27 nodes (odd), d = 0..13 covers every unordered node pair once (d = 0 the
// diagonal block), so the 351 off-diagonal node blocks are formed once and
// written to both triangles (or, PAIRS, once into the symmetric half: the
// KE_PAIRS layout).  Each thread keeps 21 double-float accumulators; the two
// threads of a row (adjacent lanes) split its nine row contractions
// sum_J dN_aJ A_iJkL per point and exchange them by shuffles.
// The per-point map streams each node's spatial gradient into shared memory
// as it is formed (the 81 gradients of a point are never live together), as a
// double-float for the contraction and in FP64 for the residual, which is
// formed in native FP64.
//
// Blocks of translation classes (element e a translate of element e mod P) can
// skip the isoparametric map (CLASS): the class table's FP64 section holds each
// class's spatial gradients and JxW, the same for every element of the class.
#pragma once
#include "fec_kernels.cuh"
#include "fec_mech_hex8.cuh"

namespace fec {

template <class Model>
struct Hex27Df64Smem {
  static constexpr int NQ = 27, A = 27, SCR2 = Model::SCR2;
  static constexpr int D_DN = 0, D_W = D_DN + NQ * A * 3, D_X = D_W + NQ, D_U = D_X + A * 3;
  // FP64 spatial gradients and JxW P of every point, read by the FP64 residual rows
  static constexpr int D_DNX = D_U + A * 3, D_P = D_DNX + NQ * A * 3;
  static constexpr int N_DOUBLE = D_P + NQ * 9;  // even
  static constexpr int F_DNX = 0, F_SCR = F_DNX + NQ * A * 3, F_A = F_SCR + NQ * SCR2;
  static constexpr int N_F2 = F_A + NQ * 45;
  static constexpr size_t BYTES = sizeof(double) * N_DOUBLE + sizeof(float2) * N_F2 + sizeof(int) * 32;
  static_assert(N_DOUBLE % 2 == 0, "float2 region alignment");
};

constexpr int HEX27_THREADS = 192;  // 162 contracting threads, padded to whole warps
// FP64 section of a hex27 class table (header: int P, FP32 offset, FP64 offset):
// per class, dNX double [27 points][27 nodes][3], then JxW double [27]
constexpr int HEX27_CLASS_BYTES = (27 * 27 * 3 + 27) * 8;

// One element by NTHR threads (thread tid), shared by the kernel below and the
// single-launch kernel of mixed element blocks.
template <class Model, bool WANT_R, bool WANT_K, int NTHR, bool CLASS = false, bool PAIRS = false>
__device__ __forceinline__ void hex27_df64_tile(const ElemArgs& g, unsigned elem, int tid, unsigned char* smem_raw) {
  constexpr int NQ = 27, A = 27, NDOF = 81, NS = Model::NS, SCR = Model::SCR, SCR2 = Model::SCR2;
  static_assert(NTHR >= 2 * NDOF, "162 contracting threads");
  using S = Hex27Df64Smem<Model>;
  using L = RefLayout<8>;
  double* dbase = reinterpret_cast<double*>(smem_raw);
  double* s_dN = dbase + S::D_DN;
  double* s_w = dbase + S::D_W;
  double* s_x = dbase + S::D_X;
  double* s_u = dbase + S::D_U;
  double* s_dNX64 = dbase + S::D_DNX;
  double* s_P64 = dbase + S::D_P;
  float2* fb = reinterpret_cast<float2*>(dbase + S::N_DOUBLE);
  float2* s_dNX = fb + S::F_DNX;
  float2* s_scr = fb + S::F_SCR;
  float2* s_A = fb + S::F_A;
  int* s_conn = reinterpret_cast<int*>(fb + S::N_F2);

  const int64_t e = elem;
  const double* cg = nullptr;  // CLASS: this element's class gradients [q][a][3], then JxW [q]
  if constexpr (CLASS) {
    const unsigned char* tab = static_cast<const unsigned char*>(g.affine);
    const int P = reinterpret_cast<const int*>(tab)[0], off64 = reinterpret_cast<const int*>(tab)[2];
    cg = reinterpret_cast<const double*>(tab + off64 + size_t(e % P) * HEX27_CLASS_BYTES);
  } else {
    for (int k = tid; k < NQ * A * 3; k += NTHR) s_dN[k] = g.ref[L::DN_OFF + k];
    for (int k = tid; k < NQ; k += NTHR) s_w[k] = g.ref[L::W_OFF + k];
  }
  if (tid < A) s_conn[tid] = g.conn[e * A + tid];
  __syncthreads();
  if (tid < A * 3) {
    const int64_t dof = int64_t(s_conn[tid / 3]) * 3 + tid % 3;
    if (!CLASS) s_x[tid] = __ldg(&g.coords[dof]);
    s_u[tid] = __ldg(&g.U[dof]);
  }
  __syncthreads();
  if (CLASS && tid < NQ) {  // the class's gradients: displacement gradient and constitutive update, FP64
    const int q = tid;
    const double* gq = cg + q * A * 3;
    double gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    float2* pdNX = s_dNX + q * A * 3;
#pragma unroll 3
    for (int a = 0; a < A; ++a) {
      double gx[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        gx[d] = __ldg(gq + a * 3 + d);
        pdNX[a * 3 + d] = df64_split(gx[d]);
        if (WANT_R) s_dNX64[(q * A + a) * 3 + d] = gx[d];
      }
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) gu[i][j] = fma(s_u[a * 3 + i], gx[j], gu[i][j]);
    }
    const double jxw = __ldg(cg + NQ * A * 3 + q);
    const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
    double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
    double P9[9], scr[SCR];
    Model::point(g.props, gu, jxw, so, sn, P9, scr);
    if (WANT_R)
#pragma unroll
      for (int m = 0; m < 9; ++m) s_P64[q * 9 + m] = P9[m];
    Model::split_scratch(scr, s_scr + q * SCR2);
  }
  if (!CLASS && tid < NQ) {  // per-point map and constitutive update, native FP64
    const int q = tid;
    const double* dN = s_dN + q * A * 3;
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll 3
    for (int a = 0; a < A; ++a)
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int k = 0; k < 3; ++k) J[d][k] = fma(s_x[a * 3 + d], dN[a * 3 + k], J[d][k]);
    const double det = det3(J);
    const double rdet = 1.0 / det;
    double Ji[3][3];
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * rdet;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * rdet;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * rdet;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * rdet;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * rdet;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * rdet;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * rdet;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * rdet;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * rdet;
    double gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    float2* pdNX = s_dNX + q * A * 3;
#pragma unroll 3
    for (int a = 0; a < A; ++a) {
      double gx[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double s = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) s = fma(dN[a * 3 + k], Ji[k][d], s);
        gx[d] = s;
        pdNX[a * 3 + d] = df64_split(s);
        if (WANT_R) s_dNX64[(q * A + a) * 3 + d] = s;
      }
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) gu[i][j] = fma(s_u[a * 3 + i], gx[j], gu[i][j]);
    }
    const double jxw = det * s_w[q];
    const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
    double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
    double P9[9], scr[SCR];
    Model::point(g.props, gu, jxw, so, sn, P9, scr);
    if (WANT_R)
#pragma unroll
      for (int m = 0; m < 9; ++m) s_P64[q * 9 + m] = P9[m];
    Model::split_scratch(scr, s_scr + q * SCR2);
  }
  __syncthreads();
  if (WANT_K) {
    for (int w = tid; w < NQ * 45; w += NTHR) {
      const int q = w / 45;
      int r1, r2;
      sym_pair(w - q * 45, r1, r2);
      s_A[w] = Model::aentry_df64(s_scr + q * SCR2, r1 / 3, r1 % 3, r2 / 3, r2 % 3);
    }
    __syncthreads();
  }
  if (tid >= 2 * NDOF) return;
  const int r = tid >> 1, cs = tid & 1;
  const int a = r / 3, i = r % 3;
  const float2 z = make_float2(0.f, 0.f);
  if (WANT_R && cs == 0) {  // residual row (a, i) in native FP64, points in order
    double R = 0.0;
    for (int q = 0; q < NQ; ++q) {
      const double* gx = s_dNX64 + (q * A + a) * 3;
      const double* P = s_P64 + q * 9 + i * 3;
      R = fma(gx[0], P[0], fma(gx[1], P[1], fma(gx[2], P[2], R)));
    }
    static_cast<double*>(g.Re)[e * NDOF + r] = R;
  }
  float2 K[21];
#pragma unroll
  for (int c = 0; c < 21; ++c) K[c] = z;
  const unsigned pm = 3u << ((threadIdx.x & 31u) & ~1u);  // this row's two lanes
#pragma unroll 1
  for (int q = 0; q < NQ; ++q) {
    const float2* dNX = s_dNX + q * A * 3;
    const float2 g0 = dNX[a * 3], g1 = dNX[a * 3 + 1], g2 = dNX[a * 3 + 2];
    if (WANT_K) {
      const float2* Aq = s_A + q * 45;
      // t_kL = sum_J dN_aJ A_iJkL: this thread forms kl = cs, cs + 2, ..., the
      // row's other thread the rest
      float2 t[9];
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const int kl = 2 * j + cs;
        float2 v = z;
        if (kl < 9)
          v = df64_dot3(g0, Aq[sym_index(3 * i, kl)], g1, Aq[sym_index(3 * i + 1, kl)], g2,
                        Aq[sym_index(3 * i + 2, kl)]);
        const float2 o = make_float2(__shfl_xor_sync(pm, v.x, 1), __shfl_xor_sync(pm, v.y, 1));
        t[2 * j] = cs ? o : v;
        if (2 * j + 1 < 9) t[2 * j + 1] = cs ? v : o;
      }
#pragma unroll
      for (int dd = 0; dd < 7; ++dd) {
        int b = a + 7 * cs + dd;
        b = b >= A ? b - A : b;
        const float2 h0 = dNX[b * 3], h1 = dNX[b * 3 + 1], h2 = dNX[b * 3 + 2];
#pragma unroll
        for (int k = 0; k < 3; ++k)
          K[dd * 3 + k] = df64_dot3_acc_lazy(K[dd * 3 + k], t[k * 3], h0, t[k * 3 + 1], h1, t[k * 3 + 2], h2);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 21; ++c) K[c] = df64_renorm(K[c]);
  if (WANT_K && PAIRS) {  // K_(a,i),(b,k) at its place in the symmetric half
    float2* Kp = static_cast<float2*>(g.Ke) + e * (A * (A + 1) / 2 * 9);
#pragma unroll
    for (int dd = 0; dd < 7; ++dd) {
      int b = a + 7 * cs + dd;
      b = b >= A ? b - A : b;
#pragma unroll
      for (int k = 0; k < 3; ++k) Kp[pair_entry(A, a, i, b, k)] = K[dd * 3 + k];
    }
  } else if (WANT_K) {
    float2* Ke = static_cast<float2*>(g.Ke) + e * (NDOF * NDOF);
#pragma unroll
    for (int dd = 0; dd < 7; ++dd) {
      const int d = 7 * cs + dd;
      int b = a + d;
      b = b >= A ? b - A : b;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        Ke[r * NDOF + b * 3 + k] = K[dd * 3 + k];
        if (d) Ke[(b * 3 + k) * NDOF + r] = K[dd * 3 + k];
      }
    }
  }
}

template <class Model, bool WANT_R, bool WANT_K, bool CLASS = false, bool PAIRS = false>
__global__ void __launch_bounds__(HEX27_THREADS, 3) mech_hex27_df64_kernel(ElemArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  hex27_df64_tile<Model, WANT_R, WANT_K, HEX27_THREADS, CLASS, PAIRS>(g, blockIdx.x, threadIdx.x, smem_raw);
}

}  // namespace fec
