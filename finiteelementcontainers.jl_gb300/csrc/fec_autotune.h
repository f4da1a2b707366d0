// fec_autotune.h -- the launch-configuration autotuner of the generic element
// kernels: threads per element (column split) and elements per CTA.
#pragma once
#include <cuda_runtime.h>
#include "fec_kernels.cuh"

namespace fec {

using TuneFn = cudaError_t (*)(const ElemArgs&, cudaStream_t);
struct TuneCandidate {
  const char* label;  // e.g. "EPB=8 CSPLIT=1"
  TuneFn fn;
};

// Launches the configuration tuned for (family, device, problem-size bucket).
// The first call for a key outside stream capture times every candidate on the
// caller's own data with CUDA events on its stream and keeps the fastest; all
// candidates compute identical results (same per-entry summation order), so
// the outputs do not depend on the choice.  Under stream capture an untuned
// key launches candidate `dflt`; FEC_AUTOTUNE=0 always launches `dflt`, and
// FEC_AUTOTUNE_CANDIDATE=i always launches candidate i.
cudaError_t tuned_launch(const char* family, const TuneCandidate* cand, int n, int dflt, const ElemArgs& a,
                         cudaStream_t s);

// One line per tuned key: family, size bucket, choice and each candidate's time.
int tuned_report(char* buf, size_t len);

}  // namespace fec
