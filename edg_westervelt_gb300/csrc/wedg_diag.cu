// Diagnostics on the device: of the source-mode run (src/solver.jl:839-958) the
// receiver values of v_h, the Westervelt energy with max|v_h| and min(1 - 2βv_h),
// the slice of v_h along a mesh line and snapshots of v_h on the point grid; and
// the error norms of src/solver.jl:774-836 (wedg_norms).
//
// They run once per step (receivers), once per record or once per run, so they
// use runtime sizes (n ≤ 8) and one thread per element or per output value; sums
// are taken in a fixed order (per block a fixed tree, then the blocks in order),
// so a run gives the same values every time.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/wedg.h"
#include "wedg_diag.h"

namespace wedg {

// v_h at each receiver: Σ_ab py[a] V[a][b] px[b] (src/solver.jl:920-925)
__global__ void k_receivers(const double *v, int E, int nv, int nrec, const int *rec_e, const double *py,
                            const double *px, double *out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  const int e = rec_e[r];
  double s = 0;
  for (int a = 0; a < nv; ++a) {
    double t = 0;
    for (int b = 0; b < nv; ++b) t = fma(v[e + (size_t)E * (a + nv * b)], px[r * nv + b], t);
    s = fma(py[r * nv + a], t, s);
  }
  out[r] = s;
}

// Per element (src/solver.jl:864-888): E_e = (h²/4) Σ_rs w_r w_s (½c²(ux² + uy²) + (½ - ⅔βv_h)v_h²)
// with ux = (2/h) P_u U S_uᵀ, uy = (2/h) S_u U P_uᵀ, v_h = P_v V P_vᵀ; max|v_h|, min(1 - 2βv_h).
// Each block reduces its elements in a fixed tree and writes one partial of each.
__global__ void __launch_bounds__(DIAG_THREADS) k_energy_elems(const double *u, const double *v, DiagBasis B,
                                                                const double *c2q, const double *bq, double *part) {
  __shared__ double sE[DIAG_THREADS], sV[DIAG_THREADS], sN[DIAG_THREADS];
  const int E = B.E, nu = B.nu, nv = B.nv, nq = B.nu;
  const int e = blockIdx.x * DIAG_THREADS + threadIdx.x;
  double Ee = 0.0, vmax = 0.0, ndmin = 1.0 / 0.0;
  if (e < E) {
    double U[8][8], V[8][8];
    for (int b = 0; b < nu; ++b)
      for (int a = 0; a < nu; ++a) U[a][b] = u[e + (size_t)E * (a + nu * b)];
    for (int b = 0; b < nv; ++b)
      for (int a = 0; a < nv; ++a) V[a][b] = v[e + (size_t)E * (a + nv * b)];
    // row contractions: US[a][s] = Σ_b U[a][b] S[s][b], UP likewise, VP[a][s] = Σ_b V[a][b] P[s][b]
    double US[8][8], UP[8][8], VP[8][8];
    for (int a = 0; a < nu; ++a)
      for (int s = 0; s < nq; ++s) {
        double x = 0, y = 0;
        for (int b = 0; b < nu; ++b) { x = fma(U[a][b], B.S[s][b], x); y = fma(U[a][b], B.P[s][b], y); }
        US[a][s] = x;
        UP[a][s] = y;
      }
    for (int a = 0; a < nv; ++a)
      for (int s = 0; s < nq; ++s) {
        double x = 0;
        for (int b = 0; b < nv; ++b) x = fma(V[a][b], B.P[s][b], x);
        VP[a][s] = x;
      }
    double sum = 0;
    for (int s = 0; s < nq; ++s)
      for (int r = 0; r < nq; ++r) {
        double ux = 0, uy = 0, vh = 0;
        for (int a = 0; a < nu; ++a) { ux = fma(B.P[r][a], US[a][s], ux); uy = fma(B.S[r][a], UP[a][s], uy); }
        for (int a = 0; a < nv; ++a) vh = fma(B.P[r][a], VP[a][s], vh);
        ux *= B.two_h;
        uy *= B.two_h;
        const size_t q = e + (size_t)E * (r + nq * s);
        const double c2 = c2q[q], be = bq[q];
        const double z = (B.w[r] * B.w[s]) * (0.5 * c2 * (ux * ux + uy * uy) + (0.5 - (2.0 / 3.0) * be * vh) * (vh * vh));
        sum += z;
        vmax = fmax(vmax, fabs(vh));
        ndmin = fmin(ndmin, 1.0 - 2.0 * be * vh);
      }
    Ee = B.hh4 * sum;
  }
  sE[threadIdx.x] = Ee;
  sV[threadIdx.x] = vmax;
  sN[threadIdx.x] = ndmin;
  __syncthreads();
  for (int w = DIAG_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sE[threadIdx.x] += sE[threadIdx.x + w];
      sV[threadIdx.x] = fmax(sV[threadIdx.x], sV[threadIdx.x + w]);
      sN[threadIdx.x] = fmin(sN[threadIdx.x], sN[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sE[0];
    part[gridDim.x + blockIdx.x] = sV[0];
    part[2 * gridDim.x + blockIdx.x] = sN[0];
  }
}

// The partials of all blocks, reduced by one block in a fixed order, into out[0..2]
__global__ void __launch_bounds__(DIAG_THREADS) k_energy_final(const double *part, int nblk, double *outE,
                                                                double *outV, double *outN) {
  __shared__ double sE[DIAG_THREADS], sV[DIAG_THREADS], sN[DIAG_THREADS];
  double Ee = 0.0, vmax = 0.0, ndmin = 1.0 / 0.0;
  for (int i = threadIdx.x; i < nblk; i += DIAG_THREADS) {
    Ee += part[i];
    vmax = fmax(vmax, part[nblk + i]);
    ndmin = fmin(ndmin, part[2 * nblk + i]);
  }
  sE[threadIdx.x] = Ee;
  sV[threadIdx.x] = vmax;
  sN[threadIdx.x] = ndmin;
  __syncthreads();
  for (int w = DIAG_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sE[threadIdx.x] += sE[threadIdx.x + w];
      sV[threadIdx.x] = fmax(sV[threadIdx.x], sV[threadIdx.x + w]);
      sN[threadIdx.x] = fmin(sN[threadIdx.x], sN[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *outE = sE[0];
    *outV = sV[0];
    *outN = sN[0];
  }
}

// Slice of v_h along the element row j0 at the local y of py: out[k nq + i] =
// Σ_b P_v[i][b] Σ_a py[a] V_{j0,k}[a][b] (src/solver.jl:914-915)
__global__ void k_slice(const double *v, DiagBasis B, int j0, const double *py, double *out) {
  const int nq = B.nu, nv = B.nv, N = B.N, E = B.E;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N * nq) return;
  const int k = g / nq, i = g - k * nq;
  const int e = j0 + N * k;
  double s = 0;
  for (int b = 0; b < nv; ++b) {
    double wb = 0;
    for (int a = 0; a < nv; ++a) wb = fma(py[a], v[e + (size_t)E * (a + nv * b)], wb);
    s = fma(B.P[i][b], wb, s);
  }
  out[g] = s;
}

// v_h on the (N nq)² point grid, column-major: G[(j nq + r) + N nq (k nq + s)] = (P_v V_{j,k} P_vᵀ)[r][s]
// (src/solver.jl:927-931)
__global__ void k_vgrid(const double *v, DiagBasis B, double *out) {
  const int nq = B.nu, nv = B.nv, N = B.N, E = B.E;
  const size_t M = (size_t)N * nq;
  const size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (g >= M * M) return;
  const size_t row = g % M, col = g / M;
  const int j = (int)(row / nq), r = (int)(row % nq), k = (int)(col / nq), s = (int)(col % nq);
  const int e = j + N * k;
  double x = 0;
  for (int a = 0; a < nv; ++a) {
    double t = 0;
    for (int b = 0; b < nv; ++b) t = fma(v[e + (size_t)E * (a + nv * b)], B.P[s][b], t);
    x = fma(B.P[r][a], t, x);
  }
  out[g] = x;
}

}  // namespace wedg

namespace wedg {

// Error norms (src/solver.jl:774-836): per element the four sums Σ W du², Σ W dv²,
// Σ W (dux² + duy²), Σ W (½c²(dux² + duy²) + ½dv²) at the u-quadrature points, with du, dv,
// dux, duy the modal differences A - B taken to the points (difference_norms) or the
// manufactured solution minus the state (_mms_errors); a fixed-order block reduction.
__global__ void __launch_bounds__(DIAG_THREADS) k_norms(NormArgs A, double *part) {
  __shared__ double sm[4][DIAG_THREADS];
  const DiagBasis &B = A.B;
  const int E = B.E, N = B.N, nu = B.nu, nv = B.nv, nq = B.nu;
  const int e = blockIdx.x * DIAG_THREADS + threadIdx.x;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  if (e < E) {
    const int j = e % N, k = e / N;
    double U[8][8], V[8][8];
    for (int b = 0; b < nu; ++b)
      for (int a = 0; a < nu; ++a) {
        const size_t l = e + (size_t)E * (a + nu * b);
        U[a][b] = A.uB ? A.uA[l] - A.uB[l] : A.uA[l];
      }
    for (int b = 0; b < nv; ++b)
      for (int a = 0; a < nv; ++a) {
        const size_t l = e + (size_t)E * (a + nv * b);
        V[a][b] = A.vB ? A.vA[l] - A.vB[l] : A.vA[l];
      }
    double US[8][8], UP[8][8], VP[8][8];
    for (int a = 0; a < nu; ++a)
      for (int s = 0; s < nq; ++s) {
        double x = 0, y = 0;
        for (int b = 0; b < nu; ++b) { x = fma(U[a][b], B.S[s][b], x); y = fma(U[a][b], B.P[s][b], y); }
        US[a][s] = x;
        UP[a][s] = y;
      }
    for (int a = 0; a < nv; ++a)
      for (int s = 0; s < nq; ++s) {
        double x = 0;
        for (int b = 0; b < nv; ++b) x = fma(V[a][b], B.P[s][b], x);
        VP[a][s] = x;
      }
    const double kxa = 2.0 * M_PI * A.kx, kya = 2.0 * M_PI * A.ky, cm = A.ctT - 1.0, vs = -A.omega * A.stT;
    for (int s = 0; s < nq; ++s)
      for (int r = 0; r < nq; ++r) {
        double uh = 0, ux = 0, uy = 0, vh = 0;
        for (int a = 0; a < nu; ++a) {
          uh = fma(B.P[r][a], UP[a][s], uh);
          ux = fma(B.P[r][a], US[a][s], ux);
          uy = fma(B.S[r][a], UP[a][s], uy);
        }
        for (int a = 0; a < nv; ++a) vh = fma(B.P[r][a], VP[a][s], vh);
        ux *= B.two_h;
        uy *= B.two_h;
        double du, dv, dux, duy;
        if (A.mms) {
          const double X = A.xloc[k + (size_t)N * s], Y = A.yloc[j + (size_t)N * r];
          const double cx = cos(kxa * X + A.px), sx = sin(kxa * X + A.px);
          const double cy = cos(kya * Y + A.py), sy = sin(kya * Y + A.py);
          const double sp = cx * sy, sp_x = -kxa * sx * sy, sp_y = kya * cx * cy;
          du = cm * sp - uh;
          dv = vs * sp - vh;
          dux = cm * sp_x - ux;
          duy = cm * sp_y - uy;
        } else {
          du = uh; dv = vh; dux = ux; duy = uy;
        }
        const double W = B.w[r] * B.w[s];
        const double g = dux * dux + duy * duy;
        acc[0] += W * (du * du);
        acc[1] += W * (dv * dv);
        acc[2] += W * g;
        acc[3] += W * (0.5 * A.c2q[e + (size_t)E * (r + nq * s)] * g + 0.5 * (dv * dv));
      }
  }
  for (int q = 0; q < 4; ++q) sm[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = DIAG_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 4; ++q) sm[q][threadIdx.x] += sm[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) part[q * gridDim.x + blockIdx.x] = sm[q][0];
}

// The four sums over all blocks, in a fixed order
__global__ void __launch_bounds__(DIAG_THREADS) k_norms_final(const double *part, int nblk, double *out) {
  __shared__ double sm[4][DIAG_THREADS];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < nblk; i += DIAG_THREADS)
    for (int q = 0; q < 4; ++q) acc[q] += part[q * nblk + i];
  for (int q = 0; q < 4; ++q) sm[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = DIAG_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 4; ++q) sm[q][threadIdx.x] += sm[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = sm[threadIdx.x][0];
}

}  // namespace wedg

namespace {

// Device buffers of one wedg_norms call, freed on every return path
struct NormBuffers {
  std::vector<void *> p;
  cudaError_t get(double **q, size_t n) {
    void *x = nullptr;
    const cudaError_t e = cudaMalloc(&x, (n ? n : 1) * sizeof(double));
    if (e == cudaSuccess) p.push_back(x);
    *q = static_cast<double *>(x);
    return e;
  }
  ~NormBuffers() {
    for (void *x : p) cudaFree(x);
  }
};

}  // namespace

extern "C" int wedg_norms(const wedg_norm_args *a, double out[4]) {
  using namespace wedg;
  if (!a || !out) return WEDG_ERR_ARGUMENT;
  const int N = a->N, nu = a->qu1, nv = a->qv1, nq = nu;
  if (N < 1 || nu < 2 || nu > 8 || !(nv == nu || nv == nu - 1) || !a->w || !a->P_u || !a->S_u || !a->err_c2 ||
      !a->uA || !a->vA || (!a->uB) != (!a->vB) || (!a->uB && (!a->xloc || !a->yloc)))
    return WEDG_ERR_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return WEDG_ERR_NO_DEVICE;
  const size_t E = (size_t)N * N, nU = E * nu * nu, nV = E * nv * nv, nC = E * nq * nq;
  NormArgs A{};
  A.B.N = N; A.B.E = (int)E; A.B.nu = nu; A.B.nv = nv;
  const double h = 1.0 / N;
  A.B.two_h = 2.0 / h;
  A.B.hh4 = h * h / 4;
  for (int i = 0; i < nq; ++i) {
    A.B.w[i] = a->w[i];
    for (int d = 0; d < nu; ++d) { A.B.P[i][d] = a->P_u[i + nq * d]; A.B.S[i][d] = a->S_u[i + nq * d]; }
  }
  A.mms = a->uB ? 0 : 1;
  A.kx = a->kx; A.ky = a->ky;
  A.omega = a->omega; A.ctT = a->ctT; A.stT = a->stT; A.px = a->px; A.py = a->py;
  NormBuffers R;
  cudaError_t ce = cudaSuccess;
  auto put = [&](const double *src, size_t n, bool state, const double **dst) {
    if (ce != cudaSuccess || !src) { *dst = nullptr; return; }
    if (state && a->where == WEDG_DEVICE) { *dst = src; return; }
    double *d = nullptr;
    ce = R.get(&d, n);
    if (ce == cudaSuccess) ce = cudaMemcpy(d, src, n * sizeof(double), cudaMemcpyHostToDevice);
    *dst = d;
  };
  put(a->uA, nU, true, &A.uA);
  put(a->vA, nV, true, &A.vA);
  put(a->uB, nU, true, &A.uB);
  put(a->vB, nV, true, &A.vB);
  put(a->err_c2, nC, false, &A.c2q);
  put(a->xloc, (size_t)N * nq, false, &A.xloc);
  put(a->yloc, (size_t)N * nq, false, &A.yloc);
  const int nblk = (int)((E + DIAG_THREADS - 1) / DIAG_THREADS);
  double *part = nullptr, *sums = nullptr;
  if (ce == cudaSuccess) ce = R.get(&part, 4 * (size_t)nblk);
  if (ce == cudaSuccess) ce = R.get(&sums, 4);
  if (ce == cudaSuccess) {
    k_norms<<<nblk, DIAG_THREADS>>>(A, part);
    k_norms_final<<<1, DIAG_THREADS>>>(part, nblk, sums);
    ce = cudaGetLastError();
  }
  double s4[4] = {0, 0, 0, 0};
  if (ce == cudaSuccess) ce = cudaMemcpy(s4, sums, sizeof s4, cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return WEDG_ERR_CUDA;
  for (int q = 0; q < 4; ++q) out[q] = (h / 2) * std::sqrt(s4[q]);
  return WEDG_OK;
}
