// Kernels of the source-mode diagnostics (wedg_diag.cu), launched by wedg_run_source.
#pragma once
#include <cuda_runtime.h>

namespace wedg {

constexpr int DIAG_THREADS = 128;

// The u-quadrature operators and mesh factors the diagnostics need (n ≤ 8).
struct DiagBasis {
  int N, E, nu, nv;
  double two_h, hh4;              // 2/h, h²/4
  double w[8], P[8][8], S[8][8];  // u-quadrature weights, P_u[i][d], S_u[i][d]; P_v = P_u[:, :nv]
};

// Inputs of the error norms: states A (and B for a difference; NULL for the manufactured solution)
struct NormArgs {
  DiagBasis B;
  const double *uA, *vA, *uB, *vB, *c2q, *xloc, *yloc;
  int mms, kx, ky;
  double omega, ctT, stT, px, py;
};

__global__ void k_receivers(const double *v, int E, int nv, int nrec, const int *rec_e, const double *py,
                            const double *px, double *out);
__global__ void k_energy_elems(const double *u, const double *v, DiagBasis B, const double *c2q, const double *bq,
                               double *part);
__global__ void k_energy_final(const double *part, int nblk, double *outE, double *outV, double *outN);
__global__ void k_slice(const double *v, DiagBasis B, int j0, const double *py, double *out);
__global__ void k_vgrid(const double *v, DiagBasis B, double *out);
__global__ void k_norms(NormArgs A, double *part);
__global__ void k_norms_final(const double *part, int nblk, double *out);

}  // namespace wedg
