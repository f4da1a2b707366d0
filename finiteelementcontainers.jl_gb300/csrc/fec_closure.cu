// fec_closure.cu -- the learned J2 closure: exact return-map batches (training
// data and the reference for its error), the MLP's training kernels (forward/backward, Adam) and
// the closure physics inside the element kernel.
#include <cmath>
#include "../../include/fec_gb300.h"
#include "fec_closure.cuh"
#include "fec_closure_physics.cuh"
#include "fec_launch.h"

namespace fec {

cudaError_t launch_mech_j2mlp(int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& a,
                              cudaStream_t s, int* launches) {
  if (elem_type != 1 || precision != 1) return cudaErrorNotSupported;  // hex8, FP32 element arithmetic
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  constexpr int EPB = 8;
  const dim3 block(24, EPB);
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  ++*launches;
  if (want_r && want_k) {
    constexpr size_t smem = mech_smem_bytes<1, J2MLP, float, EPB, true>();
    cudaError_t e = ensure_smem<mech_element_kernel<1, J2MLP, float, EPB, 1, true, true>>(smem);
    if (e != cudaSuccess) return e;
    mech_element_kernel<1, J2MLP, float, EPB, 1, true, true><<<grid, block, smem, s>>>(a);
  } else if (want_r) {
    constexpr size_t smem = mech_smem_bytes<1, J2MLP, float, EPB, false>();
    cudaError_t e = ensure_smem<mech_element_kernel<1, J2MLP, float, EPB, 1, true, false>>(smem);
    if (e != cudaSuccess) return e;
    mech_element_kernel<1, J2MLP, float, EPB, 1, true, false><<<grid, block, smem, s>>>(a);
  } else {
    constexpr size_t smem = mech_smem_bytes<1, J2MLP, float, EPB, true>();
    cudaError_t e = ensure_smem<mech_element_kernel<1, J2MLP, float, EPB, 1, false, true>>(smem);
    if (e != cudaSuccess) return e;
    mech_element_kernel<1, J2MLP, float, EPB, 1, false, true><<<grid, block, smem, s>>>(a);
  }
  return cudaGetLastError();
}

namespace {

struct J2Params {
  double p[8];  // E, nu, sigma_y, H and the derived constants (J2::fill_derived)
};

// exact J2 update of a batch of points (FP64): data generation and the error reference
__global__ void j2_points_kernel(J2Params P, int64_t n, const double* strain, const double* st_old, double* stress,
                                 double* st_new, double* tangent) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double gu[3][3];
  const double* e = strain + 6 * k;
  gu[0][0] = e[0]; gu[1][1] = e[1]; gu[2][2] = e[2];
  gu[1][2] = gu[2][1] = e[3];
  gu[0][2] = gu[2][0] = e[4];
  gu[0][1] = gu[1][0] = e[5];
  double P9[9], scr[J2::SCR];
  J2::point(P.p, gu, 1.0, st_old + 7 * k, st_new + 7 * k, P9, scr);
  const int ii[6] = {0, 1, 2, 1, 0, 0}, jj[6] = {0, 1, 2, 2, 2, 1};
  for (int m = 0; m < 6; ++m) stress[6 * k + m] = P9[ii[m] * 3 + jj[m]];
  if (tangent)
    for (int m = 0; m < 6; ++m)
      for (int q = 0; q < 6; ++q)
        tangent[36 * k + 6 * m + q] = J2::aentry(scr, ii[m], jj[m], ii[q], jj[q]) * (q >= 3 ? 2.0 : 1.0);
}

// ---- MLP training: one CTA of TS threads handles TS samples ------------------
constexpr int TS = 64;
struct MlpSmem {
  static constexpr int W = 0;                                   // MLP_PARAMS
  static constexpr int X = W + MLP_PARAMS;                      // [MLP_IN][TS]
  static constexpr int A = X + MLP_IN * TS;                     // [4][64][TS] activations
  static constexpr int Z = A + 4 * MLP_HID * TS;                // [4][64][TS] pre-activations, then deltas
  static constexpr int D = Z + 4 * MLP_HID * TS;                // [MLP_OUT][TS] output deltas
  static constexpr int N = D + MLP_OUT * TS;
  static constexpr size_t BYTES = sizeof(float) * N;
};

// Forward pass and, when `partial` is set, the backward pass of the mean squared
// error on normalised targets: per-CTA parameter gradients (summed over the
// CTA's samples in a fixed order) and the CTA's squared-error sum.
__global__ void __launch_bounds__(TS) mlp_fwd_bwd_kernel(const float* params, const float* X, const float* Y,
                                                         int64_t n, float inv_count, float* partial,
                                                         float* loss_partial, float* Yout) {
  extern __shared__ __align__(16) float sm[];
  float* sW = sm + MlpSmem::W;
  float* sX = sm + MlpSmem::X;
  float* sA = sm + MlpSmem::A;
  float* sZ = sm + MlpSmem::Z;
  float* sD = sm + MlpSmem::D;
  const int t = threadIdx.x;
  const int64_t s = int64_t(blockIdx.x) * TS + t;
  const bool live = s < n;
  for (int i = t; i < MLP_PARAMS; i += TS) sW[i] = params[i];
  for (int i = 0; i < MLP_IN; ++i) sX[i * TS + t] = live ? X[s * MLP_IN + i] : 0.f;
  __syncthreads();
  // forward
  const float* in = sX;
  int nin = MLP_IN;
  for (int l = 0; l < MLP_LAYERS - 1; ++l) {
    const float* W = sW + mlp_w_off(l);
    const float* b = sW + mlp_b_off(l);
    for (int o = 0; o < MLP_HID; ++o) {
      float z = b[o];
      for (int i = 0; i < nin; ++i) z = fmaf(W[o * nin + i], in[i * TS + t], z);
      sZ[(l * MLP_HID + o) * TS + t] = z;
      sA[(l * MLP_HID + o) * TS + t] = silu(z);
    }
    in = sA + l * MLP_HID * TS;
    nin = MLP_HID;
  }
  float err2 = 0.f;
  {
    const float* W = sW + mlp_w_off(MLP_LAYERS - 1);
    const float* b = sW + mlp_b_off(MLP_LAYERS - 1);
    for (int o = 0; o < MLP_OUT; ++o) {
      float y = b[o];
      for (int i = 0; i < MLP_HID; ++i) y = fmaf(W[o * MLP_HID + i], in[i * TS + t], y);
      if (Yout && live) Yout[s * MLP_OUT + o] = y;
      const float r = live && Y ? y - Y[s * MLP_OUT + o] : 0.f;
      err2 = fmaf(r, r, err2);
      sD[o * TS + t] = 2.f * r * inv_count;
    }
  }
  if (!partial) return;
  // backward: deltas of the hidden layers overwrite their pre-activations
  {
    const float* W = sW + mlp_w_off(MLP_LAYERS - 1);
    for (int i = 0; i < MLP_HID; ++i) {
      float g = 0.f;
      for (int o = 0; o < MLP_OUT; ++o) g = fmaf(W[o * MLP_HID + i], sD[o * TS + t], g);
      float* z = sZ + (3 * MLP_HID + i) * TS + t;
      *z = g * silu_prime(*z);
    }
  }
  for (int l = MLP_LAYERS - 2; l >= 1; --l) {
    const float* W = sW + mlp_w_off(l);
    for (int i = 0; i < MLP_HID; ++i) {
      float g = 0.f;
      for (int o = 0; o < MLP_HID; ++o) g = fmaf(W[o * MLP_HID + i], sZ[(l * MLP_HID + o) * TS + t], g);
      float* z = sZ + ((l - 1) * MLP_HID + i) * TS + t;
      *z = g * silu_prime(*z);
    }
  }
  __syncthreads();
  // per-CTA parameter gradients: dW_l[o][i] = sum_s delta_l[o][s] a_{l-1}[i][s], in sample order
  float* out = partial + int64_t(blockIdx.x) * MLP_PARAMS;
  for (int l = 0; l < MLP_LAYERS; ++l) {
    const int nin_l = mlp_dim(l), nout_l = mlp_dim(l + 1);
    const float* delta = l == MLP_LAYERS - 1 ? sD : sZ + l * MLP_HID * TS;
    const float* act = l == 0 ? sX : sA + (l - 1) * MLP_HID * TS;
    for (int w = t; w < nout_l * (nin_l + 1); w += TS) {
      const int o = w / (nin_l + 1), i = w % (nin_l + 1);
      float g = 0.f;
      if (i < nin_l)
        for (int k = 0; k < TS; ++k) g = fmaf(delta[o * TS + k], act[i * TS + k], g);
      else
        for (int k = 0; k < TS; ++k) g += delta[o * TS + k];
      if (i < nin_l)
        out[mlp_w_off(l) + o * nin_l + i] = g;
      else
        out[mlp_b_off(l) + o] = g;
    }
  }
  // the CTA's squared error, summed in thread order
  __syncthreads();
  sD[t] = err2;
  __syncthreads();
  if (t == 0) {
    float e = 0.f;
    for (int k = 0; k < TS; ++k) e += sD[k];
    loss_partial[blockIdx.x] = e;
  }
}

// Sums the per-CTA gradients in CTA order; optionally applies Adam.
__global__ void mlp_reduce_adam_kernel(float* params, float* m, float* v, const float* partial, int64_t nblocks,
                                       float* grad_out, float lr, float b1, float b2, float eps, float bc1,
                                       float bc2, const float* loss_partial, float* loss_out, float inv_count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0 && loss_out) {
    float e = 0.f;
    for (int64_t b = 0; b < nblocks; ++b) e += loss_partial[b];
    *loss_out = e * inv_count;
  }
  if (p >= MLP_PARAMS) return;
  float g = 0.f;
  for (int64_t b = 0; b < nblocks; ++b) g += partial[b * MLP_PARAMS + p];
  if (grad_out) grad_out[p] = g;
  if (m) {
    const float mm = b1 * m[p] + (1.f - b1) * g;
    const float vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    params[p] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  }
}

}  // namespace
}  // namespace fec

using fec::MlpSmem;

extern "C" {

int fec_mlp_param_count(void) { return fec::MLP_PARAMS; }

int fec_j2_points(const double* props, int64_t n, const double* strain, const double* state_old, double* stress,
                  double* state_new, double* tangent, void* stream) {
  if (!props || n < 0 || (n > 0 && (!strain || !state_old || !stress || !state_new))) return FEC_ERR_ARG;
  if (n == 0) return FEC_OK;
  fec::J2Params P;
  for (int i = 0; i < 4; ++i) P.p[i] = props[i];
  fec::J2::fill_derived(P.p);
  fec::j2_points_kernel<<<unsigned((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      P, n, strain, state_old, stress, state_new, tangent);
  return cudaGetLastError() == cudaSuccess ? FEC_OK : FEC_ERR_CUDA;
}

static int mlp_pass(const float* params, const float* X, const float* Y, int64_t n, float* scratch,
                    int64_t scratch_len, float* Yout, cudaStream_t s, int64_t* nblocks_out) {
  const int64_t nb = (n + fec::TS - 1) / fec::TS;
  if (scratch && scratch_len < nb * (fec::MLP_PARAMS + 1)) return FEC_ERR_ARG;
  if (fec::ensure_smem<fec::mlp_fwd_bwd_kernel>(MlpSmem::BYTES) != cudaSuccess) return FEC_ERR_CUDA;
  float* partial = scratch;
  float* loss_partial = scratch ? scratch + nb * fec::MLP_PARAMS : nullptr;
  fec::mlp_fwd_bwd_kernel<<<unsigned(nb), fec::TS, MlpSmem::BYTES, s>>>(
      params, X, Y, n, 1.0f / float(n * fec::MLP_OUT), partial, loss_partial, Yout);
  *nblocks_out = nb;
  return cudaGetLastError() == cudaSuccess ? FEC_OK : FEC_ERR_CUDA;
}

int fec_mlp_forward(const float* params, const float* X, int64_t n, float* Y, void* stream) {
  if (!params || !X || !Y || n <= 0) return FEC_ERR_ARG;
  int64_t nb;
  return mlp_pass(params, X, nullptr, n, nullptr, 0, Y, static_cast<cudaStream_t>(stream), &nb);
}

int fec_mlp_gradient(const float* params, const float* X, const float* Y, int64_t n, float* scratch,
                     int64_t scratch_len, float* grad, float* loss, void* stream) {
  if (!params || !X || !Y || n <= 0 || !scratch || !grad) return FEC_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int64_t nb;
  int rc = mlp_pass(params, X, Y, n, scratch, scratch_len, nullptr, s, &nb);
  if (rc) return rc;
  fec::mlp_reduce_adam_kernel<<<(fec::MLP_PARAMS + 255) / 256, 256, 0, s>>>(
      nullptr, nullptr, nullptr, scratch, nb, grad, 0.f, 0.f, 0.f, 0.f, 1.f, 1.f, scratch + nb * fec::MLP_PARAMS,
      loss, 1.0f / float(n * fec::MLP_OUT));
  return cudaGetLastError() == cudaSuccess ? FEC_OK : FEC_ERR_CUDA;
}

int fec_mlp_adam_step(float* params, float* m, float* v, const float* X, const float* Y, int64_t n, int64_t step,
                      float lr, float* scratch, int64_t scratch_len, float* loss, void* stream) {
  if (!params || !m || !v || !X || !Y || n <= 0 || !scratch || step < 1) return FEC_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int64_t nb;
  int rc = mlp_pass(params, X, Y, n, scratch, scratch_len, nullptr, s, &nb);
  if (rc) return rc;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, float(step)), bc2 = 1.f - powf(b2, float(step));
  fec::mlp_reduce_adam_kernel<<<(fec::MLP_PARAMS + 255) / 256, 256, 0, s>>>(
      params, m, v, scratch, nb, nullptr, lr, b1, b2, 1e-8f, bc1, bc2, scratch + nb * fec::MLP_PARAMS, loss,
      1.0f / float(n * fec::MLP_OUT));
  return cudaGetLastError() == cudaSuccess ? FEC_OK : FEC_ERR_CUDA;
}

}  // extern "C"
