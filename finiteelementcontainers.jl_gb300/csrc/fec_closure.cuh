// fec_closure.cuh -- the learned J2 closure: a 14-64-64-64-64-13 SiLU MLP that
// stands in for the radial-return update at plastic quadrature points.
//
// Features (all in the closure's normalised units):
//   in  : elastic trial strain e_tr = eps - eps_p_old (6, tensor components xx yy zz yz xz xy),
//         eps_p_old (6), eqps_old (1), yield flag (1)
//   out : plastic correction of the deviatoric stress, s - 2 mu dev(e_tr) (6), plastic
//         strain increment (6), eqps increment (1); the elastic trial deviator and the
//         pressure kappa tr(e_tr) are added exactly (J2 flow is deviatoric)
// Parameters are stored layer by layer, W_l row-major [out][in] then b_l, FP32
// for training; the assembly reads a BF16 copy of the weights and accumulates in
// FP32.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace fec {

constexpr int MLP_LAYERS = 5;
constexpr int MLP_IN = 14, MLP_HID = 64, MLP_OUT = 13;
__host__ __device__ constexpr int mlp_dim(int l) { return l == 0 ? MLP_IN : (l == MLP_LAYERS ? MLP_OUT : MLP_HID); }
__host__ __device__ constexpr int mlp_w_off(int l) {
  int o = 0;
  for (int k = 0; k < l; ++k) o += mlp_dim(k + 1) * mlp_dim(k) + mlp_dim(k + 1);
  return o;
}
__host__ __device__ constexpr int mlp_b_off(int l) { return mlp_w_off(l) + mlp_dim(l + 1) * mlp_dim(l); }
constexpr int MLP_PARAMS = mlp_w_off(MLP_LAYERS);

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_prime(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// Closure data the assembly reads (device memory owned by the context).
struct ClosureArgs {
  const __nv_bfloat16* W;          // MLP_PARAMS entries (weights and biases), BF16
  const float* in_mean;            // MLP_IN
  const float* in_std;
  const float* out_mean;           // MLP_OUT
  const float* out_std;
  unsigned long long* counters;    // [0] plastic points, [1] fallbacks
  float tol;                       // consistency residual threshold (relative to sigma_y)
};

// Forward pass with BF16 weights and FP32 accumulation, plus the Jacobian of the
// 6 stress outputs with respect to the 6 trial-strain inputs (forward mode:
// 6 tangent vectors carried through the layers).  x, y in physical units.
__device__ inline void mlp_eval_with_jacobian(const ClosureArgs& c, const float* x, float* y, float Jsig[6][6]) {
  float a[MLP_HID], t[MLP_HID][6];
  float xn[MLP_IN];
#pragma unroll
  for (int i = 0; i < MLP_IN; ++i) xn[i] = (x[i] - c.in_mean[i]) / c.in_std[i];
  // layer 0: tangents of the inputs are unit vectors (scaled by 1/std) for the 6 strain inputs
  for (int o = 0; o < MLP_HID; ++o) {
    const __nv_bfloat16* w = c.W + mlp_w_off(0) + o * MLP_IN;
    float z = __bfloat162float(c.W[mlp_b_off(0) + o]);
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) z = fmaf(__bfloat162float(w[i]), xn[i], z);
    const float d = silu_prime(z);
#pragma unroll
    for (int j = 0; j < 6; ++j) t[o][j] = d * __bfloat162float(w[j]) / c.in_std[j];
    a[o] = silu(z);
  }
  for (int l = 1; l < MLP_LAYERS - 1; ++l) {
    float a2[MLP_HID], t2[MLP_HID][6];
    for (int o = 0; o < MLP_HID; ++o) {
      const __nv_bfloat16* w = c.W + mlp_w_off(l) + o * MLP_HID;
      float z = __bfloat162float(c.W[mlp_b_off(l) + o]);
      float tz[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int i = 0; i < MLP_HID; ++i) {
        const float wi = __bfloat162float(w[i]);
        z = fmaf(wi, a[i], z);
#pragma unroll
        for (int j = 0; j < 6; ++j) tz[j] = fmaf(wi, t[i][j], tz[j]);
      }
      const float d = silu_prime(z);
      a2[o] = silu(z);
#pragma unroll
      for (int j = 0; j < 6; ++j) t2[o][j] = d * tz[j];
    }
    for (int o = 0; o < MLP_HID; ++o) {
      a[o] = a2[o];
#pragma unroll
      for (int j = 0; j < 6; ++j) t[o][j] = t2[o][j];
    }
  }
  // output layer (linear)
  for (int o = 0; o < MLP_OUT; ++o) {
    const __nv_bfloat16* w = c.W + mlp_w_off(MLP_LAYERS - 1) + o * MLP_HID;
    float z = __bfloat162float(c.W[mlp_b_off(MLP_LAYERS - 1) + o]);
    float tz[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = 0; i < MLP_HID; ++i) {
      const float wi = __bfloat162float(w[i]);
      z = fmaf(wi, a[i], z);
#pragma unroll
      for (int j = 0; j < 6; ++j) tz[j] = fmaf(wi, t[i][j], tz[j]);
    }
    y[o] = z * c.out_std[o] + c.out_mean[o];
    if (o < 6)
#pragma unroll
      for (int j = 0; j < 6; ++j) Jsig[o][j] = tz[j] * c.out_std[o];
  }
}

}  // namespace fec
