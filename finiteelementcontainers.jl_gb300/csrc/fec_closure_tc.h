// fec_closure_tc.h -- host-side interface of the tensor-core closure kernels.
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "fec_kernels.cuh"

namespace fec {

// Per quadrature point: stress (Voigt xx yy zz yz xz xy), 6x6 tangent
// d sigma / d eps (tensor strain components), 2 floats of padding.
constexpr int POINT_TABLE_STRIDE = 44;

struct TcClosure {
  const unsigned char* image;    // packed parameters (pack_mlp_image), device
  unsigned long long* counters;  // [0] plastic points, [1] fallbacks, [2] error flag
  float* table;                  // POINT_TABLE_STRIDE floats per point of the block
  float tol;                     // consistency threshold relative to sigma_y
};

// BF16 hi/lo operand tiles of the five layers plus the FP32 biases, layer-0
// tangent seeds and normalisation, in the layout the kernels copy to shared memory.
std::vector<unsigned char> pack_mlp_image(const float* params, const float* normalisation);

// The closure kernel: point table and new state of a hex8 block.
cudaError_t launch_j2mlp_points_tc(const ElemArgs& a, const TcClosure& cl, cudaStream_t s, int* launches);
// The FP32 hex8 element kernel forming R_e and K_e (node-rows layout) from a point table.
cudaError_t launch_point_table_hex8(bool want_r, bool want_k, const ElemArgs& a, const float* table, cudaStream_t s,
                                    int* launches);

}  // namespace fec
