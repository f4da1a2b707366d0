// fec_action.cu -- matrix-free tangent action K v (the reference's
// assemble_matrix_free_action! with stiffness_action, src/assemblers/MatrixAction.jl:9-77).
//
// One thread per quadrature point: map, displacement gradient and constitutive
// update as in the assembly kernels, then the direction gradient G = grad v and
// the action of the tangent on it without forming A (Model::action, a
// directional derivative of P), and K_q v = sum_J dN_aJ (A:G)_iJ.  The element's
// point contributions are summed in point order (the reference's
// Kv_el = Kv_el + Kv_q) into the element residual workspace, which the node
// gather then reduces in element order into the unknowns -- the same
// deterministic path as the residual.  The state is read, never written.
// FP64 blocks of translated hex8 elements (args.affine: the block's constant
// spatial gradients and JxW) skip the map and the coordinate loads (AFF).
#include <type_traits>
#include "fec_launch.h"

namespace fec {
namespace {

// Shared-memory layout (bytes) of the action kernel.
template <int ET, typename Real, int EPB, int NF>
struct ActionSmem {
  using E = Elem<ET>;
  static constexpr int A = E::NNPE, D = E::DIM, NQ = E::NQ, NDOF = NF * A;
  static constexpr bool MIXED = std::is_same<Real, float>::value && D == 3;
  static constexpr size_t REF = 0;                                          // doubles
  static constexpr size_t X = REF + 8 * size_t((RefLayout<ET>::SIZE + 1) & ~1);
  static constexpr size_t U = X + 8 * size_t(EPB * A * D);
  static constexpr size_t V = U + 8 * size_t(EPB * A * NF);
  static constexpr size_t KQ = V + 8 * size_t(EPB * A * NF);                // Real
  static constexpr size_t REFF = KQ + ((sizeof(Real) * EPB * NQ * NDOF + 7) & ~size_t(7));  // floats
  static constexpr size_t XD = REFF + 4 * size_t(MIXED ? (RefLayout<ET>::SIZE + 1) & ~1 : 0);
  static constexpr size_t CONN = XD + 4 * size_t(MIXED ? EPB * A * D : 0);  // ints
  static constexpr size_t BYTES = CONN + 4 * size_t(EPB * A);
};

template <int ET, class Model, typename Real, int EPB, bool SCALAR, bool AFF = false>
__global__ void __launch_bounds__(EPB * Elem<ET>::NQ) action_kernel(ElemArgs g, const double* V) {
  using E = Elem<ET>;
  using L = RefLayout<ET>;
  constexpr int D = E::DIM, A = E::NNPE, NQ = E::NQ, NF = SCALAR ? 1 : 3, NDOF = NF * A;
  constexpr int SCR = SCALAR ? 1 : Model::SCR;
  using S = ActionSmem<ET, Real, EPB, NF>;
  constexpr bool MIXED = S::MIXED;
  extern __shared__ __align__(16) unsigned char sm[];
  double* s_ref = reinterpret_cast<double*>(sm + S::REF);
  double* s_x = reinterpret_cast<double*>(sm + S::X);
  double* s_u = reinterpret_cast<double*>(sm + S::U);
  double* s_v = reinterpret_cast<double*>(sm + S::V);
  Real* s_kq = reinterpret_cast<Real*>(sm + S::KQ);
  float* s_reff = reinterpret_cast<float*>(sm + S::REFF);
  float* s_xd = reinterpret_cast<float*>(sm + S::XD);
  int* s_conn = reinterpret_cast<int*>(sm + S::CONN);

  const int tid = threadIdx.x, nthr = EPB * NQ;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  static_assert(!AFF || (!MIXED && NQ * A * D + NQ <= L::SIZE), "gradients and JxW in the reference area");
  if constexpr (AFF) {  // dNX [q][a][d], then JxW [q]
    const double* tg = static_cast<const double*>(g.affine);
    for (int i = tid; i < NQ * A * D + NQ; i += nthr) s_ref[i] = tg[i];
  } else {
    for (int i = tid; i < L::SIZE; i += nthr) {
      s_ref[i] = g.ref[i];
      if constexpr (MIXED) s_reff[i] = float(g.ref[i]);
    }
  }
  for (int i = tid; i < EPB * A; i += nthr) {
    const int64_t e = e0 + i / A;
    s_conn[i] = e < g.ne ? g.conn[e * A + i % A] : 0;
  }
  __syncthreads();
  if constexpr (!AFF)
    for (int i = tid; i < EPB * A * D; i += nthr) s_x[i] = g.coords[int64_t(s_conn[i / D]) * D + i % D];
  for (int i = tid; i < EPB * A * NF; i += nthr) {
    const int64_t dof = int64_t(s_conn[i / NF]) * NF + i % NF;
    s_u[i] = g.U[dof];
    s_v[i] = V[dof];
  }
  __syncthreads();
  if constexpr (MIXED) {
    for (int i = tid; i < EPB * A * D; i += nthr) {
      const int el = i / (A * D), r = i % (A * D);
      s_xd[i] = float(s_x[i] - s_x[el * A * D + r % D]);
    }
    __syncthreads();
  }
  const int el = tid / NQ, q = tid % NQ;
  const int64_t e = e0 + el;
  Real* kq = s_kq + (el * NQ + q) * NDOF;
  if (e < g.ne) {
    Real dNXr[A * D];
    const Real* dNX = dNXr;  // AFF: the block's gradients of point q, read from shared memory where used
    const double* x = s_x + el * A * D;
    double jxw;
    if constexpr (AFF) {
      dNX = s_ref + q * A * D;
      jxw = s_ref[NQ * A * D + q];
    } else if constexpr (MIXED) {
      jxw = map_point_mixed<ET>(s_ref, s_reff, q, x, s_xd + el * A * D, dNXr);
    } else {
      jxw = map_point<ET, Real>(s_ref, q, x, dNXr, nullptr);
    }
    const double* u = s_u + el * A * NF;
    const double* v = s_v + el * A * NF;
    if constexpr (SCALAR) {  // Poisson: K_q = JxW dN dN^T
      Real gv[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        Real sum = 0;
#pragma unroll
        for (int a = 0; a < A; ++a) sum = fma(Real(v[a]), dNX[a * D + d], sum);
        gv[d] = Real(jxw) * sum;
      }
#pragma unroll
      for (int a = 0; a < A; ++a) {
        Real sum = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) sum = fma(dNX[a * D + d], gv[d], sum);
        kq[a] = sum;
      }
    } else {
      Real gu[3][3], gv[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          Real su = 0, sv = 0;
#pragma unroll
          for (int a = 0; a < A; ++a) {
            su = fma(Real(u[a * 3 + i]), dNX[a * 3 + j], su);
            sv = fma(Real(v[a * 3 + i]), dNX[a * 3 + j], sv);
          }
          gu[i][j] = su;
          gv[i][j] = sv;
        }
      const double* so = Model::NS ? g.state_old + (e * NQ + q) * Model::NS : nullptr;
      Real P9[9], scr[SCR], AG[3][3];
      Model::point(g.props, gu, Real(jxw), so, nullptr, P9, scr);
      Model::action(scr, gv, AG);
#pragma unroll
      for (int a = 0; a < A; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i)
          kq[a * 3 + i] = fma(dNX[a * 3], AG[i][0], fma(dNX[a * 3 + 1], AG[i][1], dNX[a * 3 + 2] * AG[i][2]));
    }
  }
  __syncthreads();
  // element sums in point order -> residual workspace
  for (int r = tid; r < EPB * NDOF; r += nthr) {
    const int le = r / NDOF, c = r % NDOF;
    const int64_t ee = e0 + le;
    if (ee >= g.ne) continue;
    Real sum = 0;
    for (int qq = 0; qq < NQ; ++qq) sum += s_kq[(le * NQ + qq) * NDOF + c];
    static_cast<Real*>(g.Re)[ee * NDOF + c] = sum;
  }
}

template <int ET, class Model, int EPB, bool SCALAR>
cudaError_t go(int precision, const ElemArgs& a, const double* V, cudaStream_t s, int* launches) {
  if (a.ne <= 0) return cudaSuccess;
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB)), block(EPB * Elem<ET>::NQ);
  constexpr int NF = SCALAR ? 1 : 3;
  cudaError_t e;
  ++*launches;
  if (precision == 0) {
    constexpr size_t smem = ActionSmem<ET, double, EPB, NF>::BYTES;
    if constexpr (ET == 1) {
      if (a.affine) {
        if ((e = ensure_smem<action_kernel<ET, Model, double, EPB, SCALAR, true>>(smem)) != cudaSuccess) return e;
        action_kernel<ET, Model, double, EPB, SCALAR, true><<<grid, block, smem, s>>>(a, V);
        return cudaGetLastError();
      }
    }
    if ((e = ensure_smem<action_kernel<ET, Model, double, EPB, SCALAR>>(smem)) != cudaSuccess) return e;
    action_kernel<ET, Model, double, EPB, SCALAR><<<grid, block, smem, s>>>(a, V);
  } else {
    constexpr size_t smem = ActionSmem<ET, float, EPB, NF>::BYTES;
    if ((e = ensure_smem<action_kernel<ET, Model, float, EPB, SCALAR>>(smem)) != cudaSuccess) return e;
    action_kernel<ET, Model, float, EPB, SCALAR><<<grid, block, smem, s>>>(a, V);
  }
  return cudaGetLastError();
}

template <class Model>
cudaError_t by_element(int elem_type, int precision, const ElemArgs& a, const double* V, cudaStream_t s,
                       int* launches) {
  switch (elem_type) {
    case 1: return go<1, Model, 16, false>(precision, a, V, s, launches);
    case 6: return go<6, Model, 128, false>(precision, a, V, s, launches);
    case 7: return go<7, Model, 32, false>(precision, a, V, s, launches);
    case 8: return go<8, Model, 2, false>(precision, a, V, s, launches);
    default: return cudaErrorNotSupported;
  }
}

struct ScalarModel {  // the Poisson stiffness needs no constitutive state
  static constexpr int SCR = 1;
};

}  // namespace

cudaError_t launch_action(int physics, int elem_type, int precision, const ElemArgs& a, const double* V,
                          cudaStream_t s, int* launches) {
  if (precision != 0 && precision != 1) return cudaErrorNotSupported;
  switch (physics) {
    case 1:
      switch (elem_type) {
        case 1: return go<1, ScalarModel, 16, true>(precision, a, V, s, launches);
        case 2: return go<2, ScalarModel, 64, true>(precision, a, V, s, launches);
        case 6: return go<6, ScalarModel, 128, true>(precision, a, V, s, launches);
        case 7: return go<7, ScalarModel, 32, true>(precision, a, V, s, launches);
        case 8: return go<8, ScalarModel, 2, true>(precision, a, V, s, launches);
        default: return cudaErrorNotSupported;
      }
    case 2: return by_element<NeoHookean>(elem_type, precision, a, V, s, launches);
    case 3: return by_element<J2>(elem_type, precision, a, V, s, launches);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace fec
