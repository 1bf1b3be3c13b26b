// Set-up kernels of wedg_create: the packed inverses of the pinned c²-stiffness of every
// element (src/solver.jl:528-535), computed on the device from the element's c²W at the
// u-quadrature points when the caller passes no Ainv_u.
//
// One block per element, the n × n matrix (n = (q_u+1)² ≤ 64) in shared memory:
//   M = Φξᵀ diag(c²W) Φξ + Φηᵀ diag(c²W) Φη, M[0][0] += 1, with Φξ = P_u ⊗ S_u, Φη = S_u ⊗ P_u
//   (Kronecker products in numpy's `kron` index order: row p1 nq + p2, column i1 nu + i2);
//   M = L Lᵀ (Cholesky, right-looking); Li = L⁻¹ (forward substitution, a column per thread);
//   A = Liᵀ Li, written as the packed upper triangle by columns, row j(j+1)/2 + i, [row E + e].
// A pivot that is not positive sets the element's flag (the reference's cholesky throws).
#include <cuda_runtime.h>

#include "wedg_setup.h"

namespace wedg {

__global__ void k_ainv(const double *Cw, int E, int nu, const double *Pu, const double *Su, double *Ainv,
                       unsigned int *bad) {
  extern __shared__ double sh[];
  const int e = blockIdx.x;
  if (e >= E) return;
  const int nq = nu, n = nu * nu, np = nq * nq;
  double *M = sh, *Li = sh + n * n, *cw = Li + n * n, *P = cw + np, *S = P + nq * nu;
  __shared__ int fail;
  const int t = threadIdx.x, T = blockDim.x;
  if (t == 0) fail = 0;
  for (int i = t; i < np; i += T) cw[i] = Cw[(size_t)i * E + e];
  for (int i = t; i < nq * nu; i += T) { P[i] = Pu[i]; S[i] = Su[i]; }   // [p + nq d], column-major
  __syncthreads();
  // ---- assembly (upper triangle computed, mirrored)
  for (int idx = t; idx < n * n; idx += T) {
    const int i = idx % n, j = idx / n;
    if (i > j) continue;
    const int i1 = i / nu, i2 = i % nu, j1 = j / nu, j2 = j % nu;
    double s = 0.0;
    for (int p1 = 0; p1 < nq; ++p1) {
      const double pa = P[p1 + nq * i1] * P[p1 + nq * j1], sa = S[p1 + nq * i1] * S[p1 + nq * j1];
      for (int p2 = 0; p2 < nq; ++p2) {
        const double c = cw[p1 * nq + p2];
        s = fma(c, pa * (S[p2 + nq * i2] * S[p2 + nq * j2]) + sa * (P[p2 + nq * i2] * P[p2 + nq * j2]), s);
      }
    }
    if (i == 0 && j == 0) s += 1.0;
    M[i + n * j] = s;
    M[j + n * i] = s;
  }
  __syncthreads();
  // ---- Cholesky: L in the lower triangle of M
  for (int k = 0; k < n; ++k) {
    if (t == 0) {
      const double d = M[k + n * k];
      if (!(d > 0.0)) fail = 1;
      M[k + n * k] = sqrt(d > 0.0 ? d : 1.0);
    }
    __syncthreads();
    const double lkk = M[k + n * k];
    for (int i = k + 1 + t; i < n; i += T) M[i + n * k] /= lkk;
    __syncthreads();
    const int m = n - k - 1;
    for (int idx = t; idx < m * m; idx += T) {
      const int i = k + 1 + idx % m, j = k + 1 + idx / m;
      if (j <= i) M[i + n * j] = fma(-M[i + n * k], M[j + n * k], M[i + n * j]);
    }
    __syncthreads();
  }
  // ---- Li = L⁻¹ (lower triangular), one column c per thread
  for (int c = t; c < n; c += T) {
    for (int i = 0; i < c; ++i) Li[i + n * c] = 0.0;
    for (int i = c; i < n; ++i) {
      double s = (i == c) ? 1.0 : 0.0;
      for (int k = c; k < i; ++k) s = fma(-M[i + n * k], Li[k + n * c], s);
      Li[i + n * c] = s / M[i + n * i];
    }
  }
  __syncthreads();
  // ---- A = Liᵀ Li, packed upper triangle by columns
  for (int idx = t; idx < n * n; idx += T) {
    const int i = idx % n, j = idx / n;
    if (i > j) continue;
    double s = 0.0;
    for (int k = j; k < n; ++k) s = fma(Li[k + n * i], Li[k + n * j], s);
    Ainv[(size_t)(j * (j + 1) / 2 + i) * E + e] = s;
  }
  if (t == 0 && fail) atomicAdd(bad, 1u);
}

size_t ainv_smem(int nu) {
  const int n = nu * nu, nq = nu;
  return sizeof(double) * (2 * (size_t)n * n + nq * nq + 2 * nq * nu);
}

}  // namespace wedg
