// Set-up kernels of wedg_create (wedg_setup.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace wedg {

// Packed inverses of the pinned c²-stiffness of every element (one block per element);
// Cw in the device layout [(r + nq s) E + e], Pu and Su column-major (nq × nu); Ainv
// [row E + e]; *bad counts the elements whose matrix is not positive definite.
__global__ void k_ainv(const double *Cw, int E, int nu, const double *Pu, const double *Su, double *Ainv,
                       unsigned int *bad);
size_t ainv_smem(int nu);   // dynamic shared memory of k_ainv

}  // namespace wedg
