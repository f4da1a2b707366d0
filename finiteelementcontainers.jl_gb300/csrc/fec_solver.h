// fec_solver.h -- device linear algebra on the assembled CSC stiffness.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace fec {

// Symmetric matrix in CSC over the unknowns (0-based), values on the device.
struct CscSym {
  int64_t n;
  const int64_t* colptr;  // n + 1
  const int32_t* rowval;  // nnz
  const double* val;      // nnz
};

size_t pcg_scratch_doubles(int64_t n);
cudaError_t spmv_sym(const CscSym& A, const double* x, double* y, cudaStream_t s);
// Conjugate gradients for A x = b from the x passed in (Jacobi-preconditioned if
// asked); stops when ||b - A x|| <= rtol ||b|| (checked every check_every
// iterations) or after max_iter.  Synchronises the stream at the checks.
cudaError_t pcg(const CscSym& A, const double* b, double* x, double* scratch, int max_iter, double rtol,
                int check_every, bool jacobi, int* iterations, double* rel_residual, cudaStream_t s);

}  // namespace fec
