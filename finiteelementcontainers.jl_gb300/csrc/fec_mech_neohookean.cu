// fec_mech_neohookean.cu -- instantiations of the mechanics element kernel for the
// NeoHookean constitutive model.
#include "fec_launch.h"

namespace fec {
namespace {

template <int ET, int EPB, int CSPLIT, typename Real, bool R, bool K>
cudaError_t go1(const ElemArgs& a, cudaStream_t s) {
  constexpr int TPE = 3 * Elem<ET>::NNPE * CSPLIT;
  constexpr size_t smem = mech_smem_bytes<ET, NeoHookean, Real, EPB, K>();
  auto kern = mech_element_kernel<ET, NeoHookean, Real, EPB, CSPLIT, R, K>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
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

}  // namespace

cudaError_t launch_mech_neohookean(int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& a,
                           cudaStream_t s, int* launches) {
  switch (elem_type) {
    case 1: return by_prec<1, 8, 1>(precision, want_r, want_k, a, s, launches);
    case 6: return by_prec<6, 16, 1>(precision, want_r, want_k, a, s, launches);
    case 7: return by_prec<7, 8, 1>(precision, want_r, want_k, a, s, launches);
    case 8: return by_prec<8, 1, 3>(precision, want_r, want_k, a, s, launches);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace fec
