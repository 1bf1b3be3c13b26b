// Dispatch of the size-templated kernels of libwedg. Each q_u = NU - 1 is
// compiled in its own translation unit (wedg_qN.cu) so that the build runs in
// parallel; this header is the interface between them and wedg_api.cu.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include <mutex>

#include "wedg_kernels.cuh"

namespace wedg {

constexpr int MAXN = 8;    // q_u ≤ 7
constexpr int MAXQH = 12;  // q_high for q_v = 7
constexpr int MAX_DEVICES = 64;

// Runtime-sized copy of the 1D operators, packed into Basis<NU, NV> per launch.
struct BasisHost {
  int nu, nv, qh;
  double w[MAXN], P[MAXN][MAXN], S[MAXN][MAXN];
  double Pw[MAXN][MAXN];
  double El[MAXN], Er[MAXN], E1l[MAXN], E1r[MAXN];
  double E1F[MAXN];
  double Ph[MAXQH][MAXN], Wh[MAXQH][MAXQH], wh[MAXQH], PhW[MAXQH][MAXN];
  double K1[MAXN][MAXN], Q[MAXN][MAXN], ilam2[MAXN][MAXN];
};

// A launcher enqueues one kernel; it returns an error only when it could not launch (a launch
// error itself is left to the caller's cudaGetLastError)
typedef cudaError_t (*launch_fn)(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads,
                                 cudaStream_t st);
typedef void (*pack_fn)(const BasisHost &h, void *out);

typedef void (*adj_fn)(const void *basis, const Fields &F, const StageIO &S, const AdjIO &A, cudaStream_t st);

// k_adj_face; with gc2 (and gal, gbe) non-null also the coefficient derivatives
typedef void (*adj_face_fn)(const void *basis, const Fields &F, const StageIO &S, const AdjIO &A, double *gc2,
                            double *gal, double *gbe, cudaStream_t st);

// Multi-instance launches (wedg_kernels.cuh): `grid` blocks (0: one per virtual block) of
// `threads` threads; the caller sets P.tile to the kernel's elements per block (k_prep: threads,
// k_stage: stage_threads, the mass solves: (threads / 32) teams per warp)
typedef cudaError_t (*multi_fn)(const void *basis, const MultiStage &P, int grid, int threads,
                                cudaStream_t st);
typedef cudaError_t (*multi_adj_fn)(const void *basis, const MultiAdj &P, int grid, cudaStream_t st);

// k_prep over the elements [e0, e0 + blocks × threads) (clipped to the mesh)
typedef cudaError_t (*prep_fn)(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads,
                               cudaStream_t st, int e0);

struct Launchers {
  prep_fn prep = nullptr;
  launch_fn stage = nullptr, mass = nullptr;
  adj_fn adj_hats = nullptr, adj_mass = nullptr;
  adj_face_fn adj_face = nullptr;
  multi_fn prep_m = nullptr, stage_m = nullptr, mass_m = nullptr;
  multi_adj_fn adj_hats_m = nullptr, adj_mass_m = nullptr, adj_face_m = nullptr;
  pack_fn pack = nullptr;
  size_t basis_size = 0;
};

static_assert(sizeof(MultiStage) + sizeof(Basis<MAXN, MAXN>) <= 32764 &&
                  sizeof(MultiAdj) + sizeof(Basis<MAXN, MAXN>) <= 32764,
              "the arguments of a multi-instance launch exceed the kernel parameter limit");

inline int multi_grid(int grid, int total) { return grid > 0 && grid < total ? grid : total; }

template <int NU, int NV>
void pack_basis(const BasisHost &h, void *out) {
  Basis<NU, NV> &b = *static_cast<Basis<NU, NV> *>(out);
  constexpr int NQ = NU, QH = Basis<NU, NV>::QH;
  for (int i = 0; i < NQ; ++i) {
    b.w[i] = h.w[i];
    for (int d = 0; d < NU; ++d) { b.P[i][d] = h.P[i][d]; b.S[i][d] = h.S[i][d]; b.Pw[i][d] = h.Pw[i][d]; }
  }
  for (int d = 0; d < NU; ++d) {
    b.El[d] = h.El[d]; b.Er[d] = h.Er[d]; b.E1l[d] = h.E1l[d]; b.E1r[d] = h.E1r[d];
    b.E1F[d] = h.E1F[d];
    for (int c = 0; c < NU; ++c) { b.K1[d][c] = h.K1[d][c]; b.Q[d][c] = h.Q[d][c]; b.ilam2[d][c] = h.ilam2[d][c]; }
  }
  for (int i = 0; i < NU; ++i) {
    double x = 0.0;
    for (int a = 0; a < NU; ++a) x += h.Q[a][i] * h.E1F[a];
    b.QE[i] = x;
  }
  for (int r = 0; r < QH; ++r) {
    b.wh[r] = h.wh[r];
    for (int d = 0; d < NV; ++d) { b.Ph[r][d] = h.Ph[r][d]; b.PhW[r][d] = h.PhW[r][d]; }
  }
}

template <int NU, int NV>
cudaError_t launch_prep(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads,
                        cudaStream_t st, int e0) {
  k_prep<NU, NV><<<blocks, threads, 0, st>>>(*static_cast<const Basis<NU, NV> *>(basis), F, S, e0);
  return cudaSuccess;
}

// The opt-in to more than 48 KB of dynamic shared memory for kernel K, once per device: a
// function attribute belongs to the context of the device that is current when it is set, so
// every device that launches the kernel needs its own (std::call_once per device index, so
// that threads that launch at once on one device set it once)
template <class Tag, class K>
cudaError_t smem_opt_in(K kernel, size_t smem) {
  static std::once_flag once[MAX_DEVICES];
  static cudaError_t result[MAX_DEVICES];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEVICES)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  std::call_once(once[dev], [&] {
    result[dev] = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  return result[dev];
}

// k_stage keeps the element blocks in dynamic shared memory (up to 227 KB per block);
// `threads` must be stage_threads(NU, NV, FAST). blocks = 0 only sets the attribute.
template <int NU, int NV, bool FAST>
struct StageTag {};
template <int NU, int NV, bool FAST>
cudaError_t launch_stage(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads,
                         cudaStream_t st) {
  constexpr size_t smem = stage_smem(NU, NV, FAST);
  const cudaError_t e = smem_opt_in<StageTag<NU, NV, FAST>>(k_stage<NU, NV, FAST>, smem);
  if (e != cudaSuccess) return e;
  if (blocks <= 0) return cudaSuccess;
  k_stage<NU, NV, FAST><<<blocks, threads, smem, st>>>(*static_cast<const Basis<NU, NV> *>(basis), F, S);
  return cudaSuccess;
}

// The mass solve: k_cheb or k_cg, a team of threads per element (static shared memory sized
// for CHEB_THREADS). `threads` (32, 64, 96 or 128) sets the warps of a block and with them its
// elements; the grid follows from F.E, `blocks` only says whether to launch.
template <int NU, int NV>
cudaError_t launch_mass(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads,
                        cudaStream_t st) {
  if (blocks <= 0) return cudaSuccess;
  const Basis<NU, NV> &B = *static_cast<const Basis<NU, NV> *>(basis);
  threads = (threads >= 32 && threads <= CHEB_THREADS && threads % 32 == 0) ? threads : CHEB_THREADS;
  const int tpb = (threads / 32) * ChebTeam<NU, NV>::TPW;
  const int grid = (F.E + tpb - 1) / tpb;
  if (F.cg) k_cg<NU, NV><<<grid, threads, 0, st>>>(B, F, S);
  else k_cheb<NU, NV><<<grid, threads, 0, st>>>(B, F, S);
  return cudaSuccess;
}

// The adjoint kernels (wedg_adjoint.cuh): element grids of 128 threads, the mass term on the team grid
template <int NU, int NV>
void launch_adj_hats(const void *basis, const Fields &F, const StageIO &, const AdjIO &A, cudaStream_t st) {
  k_adj_hats<NU, NV><<<(F.E + ADJ_THREADS - 1) / ADJ_THREADS, ADJ_THREADS, 0, st>>>(
      *static_cast<const Basis<NU, NV> *>(basis), F, A);
}
template <int NU, int NV>
void launch_adj_mass(const void *basis, const Fields &F, const StageIO &, const AdjIO &A, cudaStream_t st) {
  constexpr int tpb = ChebTeam<NU, NV>::TPB;
  k_adj_mass<NU, NV><<<(F.E + tpb - 1) / tpb, CHEB_THREADS, 0, st>>>(*static_cast<const Basis<NU, NV> *>(basis), F,
                                                                     A);
}
template <int NU, int NV>
void launch_adj_face(const void *basis, const Fields &F, const StageIO &S, const AdjIO &A, double *gc2, double *gal,
                     double *gbe, cudaStream_t st) {
  const Basis<NU, NV> &B = *static_cast<const Basis<NU, NV> *>(basis);
  const int grid = (F.E + ADJ_THREADS - 1) / ADJ_THREADS;
  if (gc2) k_adj_face<NU, NV, true><<<grid, ADJ_THREADS, 0, st>>>(B, F, S, A, gc2, gal, gbe);
  else k_adj_face<NU, NV, false><<<grid, ADJ_THREADS, 0, st>>>(B, F, S, A, nullptr, nullptr, nullptr);
}

template <int NU, int NV>
cudaError_t launch_prep_m(const void *basis, const MultiStage &P, int grid, int threads, cudaStream_t st) {
  const int total = P.first[P.n];
  if (total <= 0) return cudaSuccess;
  k_prep_m<NU, NV><<<multi_grid(grid, total), threads, 0, st>>>(*static_cast<const Basis<NU, NV> *>(basis), P);
  return cudaSuccess;
}

template <int NU, int NV, bool FAST>
struct StageMultiTag {};
template <int NU, int NV, bool FAST>
cudaError_t launch_stage_m(const void *basis, const MultiStage &P, int grid, int, cudaStream_t st) {
  constexpr size_t smem = stage_smem(NU, NV, FAST);
  const cudaError_t e = smem_opt_in<StageMultiTag<NU, NV, FAST>>(k_stage_m<NU, NV, FAST>, smem);
  if (e != cudaSuccess) return e;
  const int total = P.first[P.n];
  if (total <= 0) return cudaSuccess;
  k_stage_m<NU, NV, FAST><<<multi_grid(grid, total), stage_threads(NU, NV, FAST), smem, st>>>(
      *static_cast<const Basis<NU, NV> *>(basis), P);
  return cudaSuccess;
}

template <int NU, int NV>
cudaError_t launch_mass_m(const void *basis, const MultiStage &P, int grid, int threads, cudaStream_t st) {
  const int total = P.first[P.n];
  if (total <= 0) return cudaSuccess;
  const Basis<NU, NV> &B = *static_cast<const Basis<NU, NV> *>(basis);
  if (P.a[0].F.cg) k_mass_m<NU, NV, true><<<multi_grid(grid, total), threads, 0, st>>>(B, P);
  else k_mass_m<NU, NV, false><<<multi_grid(grid, total), threads, 0, st>>>(B, P);
  return cudaSuccess;
}

template <int NU, int NV>
cudaError_t launch_adj_hats_m(const void *basis, const MultiAdj &P, int grid, cudaStream_t st) {
  const int total = P.first[P.n];
  if (total <= 0) return cudaSuccess;
  k_adj_hats_m<NU, NV><<<multi_grid(grid, total), ADJ_THREADS, 0, st>>>(*static_cast<const Basis<NU, NV> *>(basis),
                                                                         P);
  return cudaSuccess;
}

template <int NU, int NV>
cudaError_t launch_adj_mass_m(const void *basis, const MultiAdj &P, int grid, cudaStream_t st) {
  const int total = P.first[P.n];
  if (total <= 0) return cudaSuccess;
  k_adj_mass_m<NU, NV><<<multi_grid(grid, total), CHEB_THREADS, 0, st>>>(*static_cast<const Basis<NU, NV> *>(basis),
                                                                          P);
  return cudaSuccess;
}

// PARAMS when the instances pass coefficient gradients (all or none of them)
template <int NU, int NV>
cudaError_t launch_adj_face_m(const void *basis, const MultiAdj &P, int grid, cudaStream_t st) {
  const int total = P.first[P.n];
  if (total <= 0) return cudaSuccess;
  const Basis<NU, NV> &B = *static_cast<const Basis<NU, NV> *>(basis);
  if (P.a[0].gc2) k_adj_face_m<NU, NV, true><<<multi_grid(grid, total), ADJ_THREADS, 0, st>>>(B, P);
  else k_adj_face_m<NU, NV, false><<<multi_grid(grid, total), ADJ_THREADS, 0, st>>>(B, P);
  return cudaSuccess;
}

template <int NU, int NV>
Launchers make_launchers(bool fast) {
  Launchers L;
  L.prep_m = launch_prep_m<NU, NV>;
  L.stage_m = fast ? launch_stage_m<NU, NV, true> : launch_stage_m<NU, NV, false>;
  L.mass_m = launch_mass_m<NU, NV>;
  L.adj_hats_m = launch_adj_hats_m<NU, NV>;
  L.adj_mass_m = launch_adj_mass_m<NU, NV>;
  L.adj_face_m = launch_adj_face_m<NU, NV>;
  L.adj_hats = launch_adj_hats<NU, NV>;
  L.adj_mass = launch_adj_mass<NU, NV>;
  L.adj_face = launch_adj_face<NU, NV>;
  L.prep = launch_prep<NU, NV>;
  L.mass = launch_mass<NU, NV>;
  L.stage = fast ? launch_stage<NU, NV, true> : launch_stage<NU, NV, false>;
  L.pack = pack_basis<NU, NV>;
  L.basis_size = sizeof(Basis<NU, NV>);
  return L;
}

// defined in wedg_q1.cu ... wedg_q7.cu (NU = q_u + 1)
Launchers launchers_q1(int nv, bool fast);
Launchers launchers_q2(int nv, bool fast);
Launchers launchers_q3(int nv, bool fast);
Launchers launchers_q4(int nv, bool fast);
Launchers launchers_q5(int nv, bool fast);
Launchers launchers_q6(int nv, bool fast);
Launchers launchers_q7(int nv, bool fast);

}  // namespace wedg
