// fec_closure_physics.cuh -- the J2 physics whose plastic points are served by
// the learned closure: trial state, completion from the network's outputs with
// the consistency check, and the exact radial return as fallback.
#pragma once
#include <cmath>
#include "fec_closure.cuh"
#include "fec_kernels.cuh"

namespace fec {

// Voigt index of tensor component (i, J): xx yy zz yz xz xy
__host__ __device__ constexpr int voigt(int i, int j) {
  return i == j ? i : (i + j == 3 ? 3 : (i + j == 2 ? 4 : 5));
}

// 6x6 tangent C6[m][n] = d sigma_m / d eps_n (tensor strain components) from a
// 9x9 A_iJkL accessor with minor symmetry: shear columns count both (k,L), (L,k).
template <class F>
__device__ inline void tangent6_from(F aentry, float* C6) {
  const int ii[6] = {0, 1, 2, 1, 0, 0}, jj[6] = {0, 1, 2, 2, 2, 1};
  for (int m = 0; m < 6; ++m)
    for (int n = 0; n < 6; ++n) C6[m * 6 + n] = aentry(ii[m], jj[m], ii[n], jj[n]) * (n >= 3 ? 2.f : 1.f);
}

// J2 with its radial return replaced at plastic points by the MLP closure;
// elastic points and points failing the consistency check use the exact update.
struct J2MLP {
  static constexpr bool USES_CLOSURE = true;
  static constexpr bool USES_TABLE = false;
  static constexpr int NS = 7;
  static constexpr int SCR = 36;  // JxW-scaled 6x6 tangent d sigma / d eps

  template <typename Real>
  __device__ static void exact(const double* props, Real gu[3][3], Real jxw, const double* st_old, double* st_new,
                               Real* P9, Real* scr) {
    Real s13[J2::SCR];
    J2::point(props, gu, jxw, st_old, st_new, P9, s13);
    // the consistent tangent in Voigt form, d sigma_m / d eps_n (tensor strain
    // components): (kap' - mt'/3) [m,n normal] + mt' I_mn (1/2 for shear m = n)
    // - mb' n_m n_n, shear columns counting both (k,L) and (L,k)
    const int ii[6] = {0, 1, 2, 1, 0, 0}, jj[6] = {0, 1, 2, 2, 2, 1};
    const Real ca = s13[9] - s13[10] / Real(3), mt = s13[10], mb = s13[11];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const Real nm = s13[ii[m] * 3 + jj[m]];
#pragma unroll
      for (int n = 0; n < 6; ++n) {
        const Real nn = s13[ii[n] * 3 + jj[n]];
        Real c = -mb * nm * nn;
        if (m < 3 && n < 3) c += ca;
        if (m == n) c += m < 3 ? mt : Real(0.5) * mt;
        scr[m * 6 + n] = n >= 3 ? Real(2) * c : c;
      }
    }
  }

  // Trial state of a point: e_tr = eps - eps_p_old, the network's input row x
  // (physical units) and whether the trial stress violates the yield condition.
  // FP32 arithmetic (the closure serves the FP32-element variant).
  template <typename Real>
  __device__ static bool trial(const double* props, Real gu[3][3], const double* st_old, float etr[6], float x[MLP_IN]) {
    const float E = float(props[0]), nu = float(props[1]), sy = float(props[2]), Hh = float(props[3]);
    const float mu = E / (2 * (1 + nu));
    const int ii[6] = {0, 1, 2, 1, 0, 0}, jj[6] = {0, 1, 2, 2, 2, 1};
#pragma unroll
    for (int m = 0; m < 6; ++m) etr[m] = 0.5f * (float(gu[ii[m]][jj[m]]) + float(gu[jj[m]][ii[m]])) - float(st_old[m]);
    const float tr = etr[0] + etr[1] + etr[2];
    float sn2 = 0;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const float dev = 2 * mu * (etr[m] - (m < 3 ? tr / 3.0f : 0.0f));
      sn2 += (m < 3 ? 1.0f : 2.0f) * dev * dev;
    }
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      x[m] = etr[m];
      x[6 + m] = float(st_old[m]);
    }
    x[12] = float(st_old[6]);
    x[13] = 1.0f;
    return sqrtf(sn2) - float(sqrt(2.0 / 3.0)) * (sy + Hh * float(st_old[6])) > 0;
  }

  // Completes a plastic point from the network's outputs y (physical units) and
  // the Jacobian Js of its 6 stress outputs with respect to e_tr.  The network
  // predicts the plastic correction of the deviatoric stress; the elastic trial
  // deviator 2 mu dev(e_tr) and the pressure kappa tr(e_tr) are exact (J2 plastic
  // flow is deviatoric, so tr(eps_e) = tr(e_tr)).  Returns false, writing
  // nothing, when the predicted stress misses the updated yield surface by more
  // than tol * sigma_y: the caller then applies the exact update.
  template <typename Real>
  __device__ static bool finish(const double* props, const float etr[6], float tol, float y[MLP_OUT],
                                float Js[6][6], Real jxw, const double* st_old, double* st_new, Real* P9, Real* scr) {
    const float E = float(props[0]), nu = float(props[1]), sy = float(props[2]), Hh = float(props[3]);
    const float mu = E / (2 * (1 + nu));
    const float tr = etr[0] + etr[1] + etr[2];
    const float mu2 = 2 * mu;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      y[m] += mu2 * (etr[m] - (m < 3 ? tr / 3.0f : 0.0f));
#pragma unroll
      for (int n = 0; n < 6; ++n) Js[m][n] += mu2 * ((m == n ? 1.f : 0.f) - (m < 3 && n < 3 ? 1.f / 3.f : 0.f));
    }
    const float kap = E / (3 * (1 - 2 * nu));
    const float p = kap * tr;
    // consistency: the predicted stress must lie on the updated yield surface
    const float eqps_new = float(st_old[6]) + y[12];
    const float trs = y[0] + y[1] + y[2];
    float d2 = 0;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const float dev = y[m] - (m < 3 ? trs / 3.0f : 0.0f);
      d2 += (m < 3 ? 1.0f : 2.0f) * dev * dev;
    }
    const float f = sqrtf(d2) - float(sqrt(2.0 / 3.0)) * (sy + Hh * eqps_new);
    if (!(fabsf(f) <= tol * sy)) return false;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P9[i * 3 + j] = jxw * Real(y[voigt(i, j)] + (i == j ? p : 0.f));
    if (st_new) {
#pragma unroll
      for (int m = 0; m < 7; ++m) st_new[m] = st_old[m] + double(y[6 + m]);
    }
#pragma unroll
    for (int m = 0; m < 6; ++m)
#pragma unroll
      for (int n = 0; n < 6; ++n) scr[m * 6 + n] = jxw * Real(Js[m][n] + (m < 3 && n < 3 ? kap : 0.f));
    return true;
  }

  // The whole point with the network evaluated by this thread (CUDA cores).
  template <typename Real>
  __device__ static void point_closure(const void* closure, const double* props, Real gu[3][3], Real jxw,
                                       const double* st_old, double* st_new, Real* P9, Real* scr) {
    const ClosureArgs& c = *static_cast<const ClosureArgs*>(closure);
    float etr[6];
    float x[MLP_IN], y[MLP_OUT], Js[6][6];
    if (!trial(props, gu, st_old, etr, x)) {  // elastic: exact and cheap
      exact(props, gu, jxw, st_old, st_new, P9, scr);
      return;
    }
    atomicAdd(&c.counters[0], 1ull);
    mlp_eval_with_jacobian(c, x, y, Js);
    if (!finish(props, etr, c.tol, y, Js, jxw, st_old, st_new, P9, scr)) {
      atomicAdd(&c.counters[1], 1ull);
      exact(props, gu, jxw, st_old, st_new, P9, scr);
    }
  }

  template <typename Real>
  __device__ static Real aentry(const Real* scr, int i, int J, int k, int L) {
    return scr[voigt(i, J) * 6 + voigt(k, L)] * (k == L ? Real(1) : Real(0.5));
  }
  template <typename Real>
  __device__ static void aentries(const Real* scr, int i, Real* out) {
#pragma unroll
    for (int J = 0; J < 3; ++J)
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int L = 0; L < 3; ++L) out[J * 9 + k * 3 + L] = aentry(scr, i, J, k, L);
  }
  // unused: the closure needs ElemArgs::closure
  template <typename Real>
  __device__ static void point(const double*, Real (*)[3], Real, const double*, double*, Real*, Real*) {}
};

}  // namespace fec
