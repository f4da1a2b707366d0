// fec_mech_j2.cu -- instantiations of the mechanics element kernel for the
// J2 constitutive model.
#include <cstdlib>
#include <cstdio>
#include <type_traits>
#include "fec_autotune.h"
#include "fec_launch.h"
#include "fec_mech_hex27.cuh"
#include "fec_mech_hex8.cuh"

namespace fec {
namespace {

template <int ET, int EPB, int CSPLIT, typename Real, bool R, bool K>
cudaError_t go1(const ElemArgs& a, cudaStream_t s) {
  constexpr int TPE = 3 * Elem<ET>::NNPE * CSPLIT;
  constexpr size_t smem = mech_smem_bytes<ET, J2, Real, EPB, K>();
  auto kern = mech_element_kernel<ET, J2, Real, EPB, CSPLIT, R, K>;
  cudaError_t err = ensure_smem<mech_element_kernel<ET, J2, Real, EPB, CSPLIT, R, K>>(smem);
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

// Autotuned generic kernels: elements per CTA for tet4/tet10, column split
// (threads per element) for hex27.
template <int ET, typename Real, bool R, bool K>
cudaError_t tuned1(const ElemArgs& a, cudaStream_t s) {
  constexpr const char* P = std::is_same<Real, double>::value ? "fp64" : "fp32_element";
  char fam[96];
  snprintf(fam, sizeof fam, "j2/%s/%s/%s", ET == 6 ? "tet4" : (ET == 7 ? "tet10" : "hex27"), P,
           R && K ? "R+K" : (R ? "R" : "K"));
  if constexpr (ET == 6) {
    static const TuneCandidate c[] = {{"EPB=8", go1<6, 8, 1, Real, R, K>}, {"EPB=16", go1<6, 16, 1, Real, R, K>},
                                      {"EPB=32", go1<6, 32, 1, Real, R, K>}};
    return tuned_launch(fam, c, 3, 1, a, s);
  } else if constexpr (ET == 7) {
    static const TuneCandidate c[] = {{"EPB=4", go1<7, 4, 1, Real, R, K>}, {"EPB=8", go1<7, 8, 1, Real, R, K>},
                                      {"EPB=16", go1<7, 16, 1, Real, R, K>}};
    return tuned_launch(fam, c, 3, 1, a, s);
  } else {
    static const TuneCandidate c[] = {{"EPB=1 CSPLIT=3", go1<8, 1, 3, Real, R, K>},
                                      {"EPB=2 CSPLIT=3", go1<8, 2, 3, Real, R, K>},
                                      {"EPB=1 CSPLIT=9", go1<8, 1, 9, Real, R, K>}};
    return tuned_launch(fam, c, 3, 0, a, s);
  }
}

template <int ET>
cudaError_t tuned(int precision, bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (precision != 0 && precision != 1) return cudaErrorNotSupported;
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (precision == 0) {
    if (want_r && want_k) return tuned1<ET, double, true, true>(a, s);
    if (want_r) return tuned1<ET, double, true, false>(a, s);
    return tuned1<ET, double, false, true>(a, s);
  }
  if (want_r && want_k) return tuned1<ET, float, true, true>(a, s);
  if (want_r) return tuned1<ET, float, true, false>(a, s);
  return tuned1<ET, float, false, true>(a, s);
}

template <typename Real, int EPB, bool R, bool K>
cudaError_t hex8_1(const ElemArgs& a, cudaStream_t s) {
  constexpr size_t smem = Hex8Smem<J2, Real, EPB>::BYTES;
  auto kern = mech_hex8_sym_kernel<J2, Real, EPB, R, K>;
  cudaError_t err = ensure_smem<mech_hex8_sym_kernel<J2, Real, EPB, R, K>>(smem);
  if (err != cudaSuccess) return err;
  const dim3 block(12, EPB);
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  kern<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

template <int EPB, bool R, bool K>
cudaError_t hex8_df64_1(const ElemArgs& a, cudaStream_t s) {
  constexpr size_t smem = Hex8Df64Smem<J2, EPB>::BYTES;
  const dim3 grid(unsigned((a.ne + EPB - 1) / EPB));
  cudaError_t err;
  if ((err = ensure_smem<mech_hex8_df64_kernel<J2, EPB, R, K>>(smem)) != cudaSuccess) return err;
  mech_hex8_df64_kernel<J2, EPB, R, K><<<grid, dim3(24, EPB), smem, s>>>(a);
  return cudaGetLastError();
}

template <bool R, bool K>
cudaError_t hex8_df64_ws_1(const ElemArgs& a, cudaStream_t s) {
  cudaError_t err;
  if ((err = ensure_smem<mech_hex8_df64_ws_kernel<J2, R, K>>(ws::Layout<J2>::SMEM)) != cudaSuccess) return err;
  const int64_t tiles = (a.ne + ws::EPB - 1) / ws::EPB;
  const int64_t sms = num_sms();
  const unsigned grid = unsigned(tiles < sms ? tiles : sms);
  mech_hex8_df64_ws_kernel<J2, R, K><<<grid, ws::NTHR, ws::Layout<J2>::SMEM, s>>>(a);
  return cudaGetLastError();
}

// FP64 hex8: the warp-specialised persistent kernel, or with FEC_HEX8_DF64=tile
// the one-tile-per-CTA kernel (bitwise the same results)
template <int EPB>
cudaError_t hex8_df64(bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (!hex8_df64_tile_kernel()) {
    if (want_r && want_k) return hex8_df64_ws_1<true, true>(a, s);
    if (want_r) return hex8_df64_ws_1<true, false>(a, s);
    return hex8_df64_ws_1<false, true>(a, s);
  }
  if (want_r && want_k) return hex8_df64_1<EPB, true, true>(a, s);
  if (want_r) return hex8_df64_1<EPB, true, false>(a, s);
  return hex8_df64_1<EPB, false, true>(a, s);
}

template <bool R, bool K, bool CLASS, bool PAIRS>
cudaError_t hex27_df64_2(const ElemArgs& a, cudaStream_t s) {
  constexpr size_t smem = Hex27Df64Smem<J2>::BYTES;
  cudaError_t err;
  if ((err = ensure_smem<mech_hex27_df64_kernel<J2, R, K, CLASS, PAIRS>>(smem)) != cudaSuccess) return err;
  mech_hex27_df64_kernel<J2, R, K, CLASS, PAIRS><<<unsigned(a.ne), HEX27_THREADS, smem, s>>>(a);
  return cudaGetLastError();
}

// CLASS: a block of translation classes (the class's gradients); PAIRS: the
// stiffness into the symmetric half (args.ke_pairs)
template <bool R, bool K>
cudaError_t hex27_df64_1(const ElemArgs& a, cudaStream_t s) {
  const bool cls = a.affine && class_tc_enabled();
  if (K && a.ke_pairs) return cls ? hex27_df64_2<R, K, true, true>(a, s) : hex27_df64_2<R, K, false, true>(a, s);
  return cls ? hex27_df64_2<R, K, true, false>(a, s) : hex27_df64_2<R, K, false, false>(a, s);
}

cudaError_t hex27_df64(bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (want_r && want_k) return hex27_df64_1<true, true>(a, s);
  if (want_r) return hex27_df64_1<true, false>(a, s);
  return hex27_df64_1<false, true>(a, s);
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
  constexpr size_t smem = Hex8Smem<J2, float, EPB>::BYTES;
  auto kern = mech_hex8_rows2_kernel<J2, EPB, R, K>;
  cudaError_t err = ensure_smem<mech_hex8_rows2_kernel<J2, EPB, R, K>>(smem);
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

cudaError_t launch_mech_j2(int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& a,
                           cudaStream_t s, int* launches) {
  switch (elem_type) {
    case 1:
      if (precision == 0 && a.affine && !fp64_native() && hex8_affine_enabled()) {
        if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
        return launch_hex8_affine_tc(3, want_r, want_k, a, s, launches);
      }
      if (precision == 0)
        return fp64_native() ? hex8<double, 8>(want_r, want_k, a, s, launches)
                             : hex8_df64<8>(want_r, want_k, a, s, launches);
      if (precision == 1) return hex8_f32<16>(want_r, want_k, a, s, launches);
      return cudaErrorNotSupported;
    case 6: return tuned<6>(precision, want_r, want_k, a, s, launches);
    case 7:
      if (class_tc_runs(3, 7, precision, want_r, want_k, a.affine != nullptr))
        return launch_class_tc(3, 7, precision, want_r, want_k, a, s, launches);
      return tuned<7>(precision, want_r, want_k, a, s, launches);
    case 8:
      if (class_tc_runs(3, 8, precision, want_r, want_k, a.affine != nullptr))
        return launch_class_tc(3, 8, precision, want_r, want_k, a, s, launches);
      if (precision == 1 && want_k && !hex27_on_cuda_cores())
        return launch_hex27_tc(3, want_r, want_k, a, s, launches);
      if (precision == 0 && !fp64_native()) return hex27_df64(want_r, want_k, a, s, launches);
      return tuned<8>(precision, want_r, want_k, a, s, launches);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace fec
