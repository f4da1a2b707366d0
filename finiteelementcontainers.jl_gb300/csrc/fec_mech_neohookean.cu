// fec_mech_neohookean.cu -- instantiations of the mechanics element kernel for the
// NeoHookean constitutive model.
#include <cstdlib>
#include "fec_launch.h"
#include "fec_mech_hex8.cuh"

namespace fec {
namespace {

template <int ET, int EPB, int CSPLIT, typename Real, bool R, bool K>
cudaError_t go1(const ElemArgs& a, cudaStream_t s) {
  constexpr int TPE = 3 * Elem<ET>::NNPE * CSPLIT;
  constexpr size_t smem = mech_smem_bytes<ET, NeoHookean, Real, EPB, K>();
  auto kern = mech_element_kernel<ET, NeoHookean, Real, EPB, CSPLIT, R, K>;
  cudaError_t err = ensure_smem<mech_element_kernel<ET, NeoHookean, Real, EPB, CSPLIT, R, K>>(smem);
  if (err != cudaSuccess) return err;
  const dim3 block(TPE, EPB);
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  kern<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

template <int ET, int EPB, int CSPLIT, typename Real>
cudaError_t go(bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (want_r && want_k) return go1<ET, EPB, CSPLIT, Real, true, true>(a, s);
  if (want_r) return go1<ET, EPB, CSPLIT, Real, true, false>(a, s);
  return go1<ET, EPB, CSPLIT, Real, false, true>(a, s);
}

template <int ET, int EPB, int CSPLIT>
cudaError_t by_prec(int precision, bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (precision == 0) return go<ET, EPB, CSPLIT, double>(want_r, want_k, a, s, launches);
  if (precision == 1) return go<ET, EPB, CSPLIT, float>(want_r, want_k, a, s, launches);
  return cudaErrorNotSupported;
}

template <typename Real, int EPB, bool R, bool K>
cudaError_t hex8_1(const ElemArgs& a, cudaStream_t s) {
  constexpr size_t smem = Hex8Smem<NeoHookean, Real, EPB>::BYTES;
  auto kern = mech_hex8_sym_kernel<NeoHookean, Real, EPB, R, K>;
  cudaError_t err = ensure_smem<mech_hex8_sym_kernel<NeoHookean, Real, EPB, R, K>>(smem);
  if (err != cudaSuccess) return err;
  const dim3 block(12, EPB);
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  kern<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

template <int EPB, bool R, bool K>
cudaError_t hex8_df64_1(const ElemArgs& a, cudaStream_t s) {
  constexpr size_t smem = Hex8Df64Smem<NeoHookean, EPB>::BYTES;
  auto kern = mech_hex8_df64_kernel<NeoHookean, EPB, R, K>;
  cudaError_t err = ensure_smem<mech_hex8_df64_kernel<NeoHookean, EPB, R, K>>(smem);
  if (err != cudaSuccess) return err;
  const dim3 block(12, EPB);
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  kern<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

template <int EPB>
cudaError_t hex8_df64(bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (want_r && want_k) return hex8_df64_1<EPB, true, true>(a, s);
  if (want_r) return hex8_df64_1<EPB, true, false>(a, s);
  return hex8_df64_1<EPB, false, true>(a, s);
}

// FP64 hex8: the contraction runs in df64 on the FP32 pipes unless
// FEC_FP64_CONTRACTION=native selects the all-FP64 kernel.
bool fp64_native() {
  static const bool v = [] {
    const char* e = getenv("FEC_FP64_CONTRACTION");
    return e && e[0] == 'n';
  }();
  return v;
}

template <int EPB, bool R, bool K>
cudaError_t hex8_f32_1(const ElemArgs& a, cudaStream_t s) {
  constexpr size_t smem = Hex8Smem<NeoHookean, float, EPB>::BYTES;
  auto kern = mech_hex8_rows2_kernel<NeoHookean, EPB, R, K>;
  cudaError_t err = ensure_smem<mech_hex8_rows2_kernel<NeoHookean, EPB, R, K>>(smem);
  if (err != cudaSuccess) return err;
  const dim3 block(12, EPB);
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  kern<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

template <int EPB>
cudaError_t hex8_f32(bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (want_r && want_k) return hex8_f32_1<EPB, true, true>(a, s);
  if (want_r) return hex8_f32_1<EPB, true, false>(a, s);
  return hex8_f32_1<EPB, false, true>(a, s);
}

template <typename Real, int EPB>
cudaError_t hex8(bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (want_r && want_k) return hex8_1<Real, EPB, true, true>(a, s);
  if (want_r) return hex8_1<Real, EPB, true, false>(a, s);
  return hex8_1<Real, EPB, false, true>(a, s);
}

}  // namespace

cudaError_t launch_mech_neohookean(int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& a,
                           cudaStream_t s, int* launches) {
  switch (elem_type) {
    case 1:
      if (precision == 0)
        return fp64_native() ? hex8<double, 8>(want_r, want_k, a, s, launches)
                             : hex8_df64<8>(want_r, want_k, a, s, launches);
      if (precision == 1) return hex8_f32<16>(want_r, want_k, a, s, launches);
      return cudaErrorNotSupported;
    case 6: return by_prec<6, 16, 1>(precision, want_r, want_k, a, s, launches);
    case 7: return by_prec<7, 8, 1>(precision, want_r, want_k, a, s, launches);
    case 8: return by_prec<8, 1, 3>(precision, want_r, want_k, a, s, launches);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace fec
