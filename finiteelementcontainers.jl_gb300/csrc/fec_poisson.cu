// fec_poisson.cu -- instantiations of the Poisson element kernel.
#include <type_traits>
#include "fec_launch.h"

namespace fec {
namespace {

template <int ET, int EPB, typename Real>
cudaError_t go(bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  constexpr int TPE = Elem<ET>::NNPE;
  if (a.ne <= 0) return cudaSuccess;
  const dim3 block(TPE, EPB);
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  if constexpr (ET == 1 && std::is_same<Real, double>::value) {
    if (a.affine) {  // a block of translated elements: its gradients and JxW from the affine table
      ElemArgs b = a;
      b.affine = static_cast<const unsigned char*>(a.affine) + hex8_affine_grad_offset();
      if (want_r && want_k)
        poisson_element_kernel<ET, Real, EPB, true, true, true><<<grid, block, 0, s>>>(b);
      else if (want_r)
        poisson_element_kernel<ET, Real, EPB, true, false, true><<<grid, block, 0, s>>>(b);
      else if (want_k)
        poisson_element_kernel<ET, Real, EPB, false, true, true><<<grid, block, 0, s>>>(b);
      else
        return cudaSuccess;
      ++*launches;
      return cudaGetLastError();
    }
  }
  if (want_r && want_k)
    poisson_element_kernel<ET, Real, EPB, true, true><<<grid, block, 0, s>>>(a);
  else if (want_r)
    poisson_element_kernel<ET, Real, EPB, true, false><<<grid, block, 0, s>>>(a);
  else if (want_k)
    poisson_element_kernel<ET, Real, EPB, false, true><<<grid, block, 0, s>>>(a);
  else
    return cudaSuccess;
  ++*launches;
  return cudaGetLastError();
}

template <int ET, int EPB>
cudaError_t by_prec(int precision, bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (precision == 0) return go<ET, EPB, double>(want_r, want_k, a, s, launches);
  if (precision == 1) return go<ET, EPB, float>(want_r, want_k, a, s, launches);
  return cudaErrorNotSupported;
}

}  // namespace

cudaError_t launch_poisson(int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& a,
                           cudaStream_t s, int* launches) {
  switch (elem_type) {
    case 1: return by_prec<1, 16>(precision, want_r, want_k, a, s, launches);
    case 2: return by_prec<2, 64>(precision, want_r, want_k, a, s, launches);
    case 6: return by_prec<6, 32>(precision, want_r, want_k, a, s, launches);
    case 7: return by_prec<7, 16>(precision, want_r, want_k, a, s, launches);
    case 8: return by_prec<8, 1>(precision, want_r, want_k, a, s, launches);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace fec
