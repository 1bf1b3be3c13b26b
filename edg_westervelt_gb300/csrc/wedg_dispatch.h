// Dispatch of the size-templated kernels of libwedg. Each q_u = NU - 1 is
// compiled in its own translation unit (wedg_qN.cu) so that the build runs in
// parallel; this header is the interface between them and wedg_api.cu.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "wedg_kernels.cuh"

namespace wedg {

constexpr int MAXN = 8;    // q_u ≤ 7
constexpr int MAXQH = 12;  // q_high for q_v = 7

// Runtime-sized copy of the 1D operators, packed into Basis<NU, NV> per launch.
struct BasisHost {
  int nu, nv, qh;
  double w[MAXN], P[MAXN][MAXN], S[MAXN][MAXN];
  double Pw[MAXN][MAXN];
  double El[MAXN], Er[MAXN], E1l[MAXN], E1r[MAXN];
  double ElA[MAXN], E1D[MAXN], E1F[MAXN];
  double Ph[MAXQH][MAXN], Wh[MAXQH][MAXQH], wh[MAXQH], PhW[MAXQH][MAXN];
  double K1[MAXN][MAXN], Q[MAXN][MAXN], ilam2[MAXN][MAXN];
};

typedef void (*launch_fn)(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads,
                          cudaStream_t st);
typedef void (*pack_fn)(const BasisHost &h, void *out);

typedef void (*adj_fn)(const void *basis, const Fields &F, const StageIO &S, const AdjIO &A, cudaStream_t st);

// k_adj_face; with gc2 (and gal, gbe) non-null also the coefficient derivatives
typedef void (*adj_face_fn)(const void *basis, const Fields &F, const StageIO &S, const AdjIO &A, double *gc2,
                            double *gal, double *gbe, cudaStream_t st);

struct Launchers {
  launch_fn prep = nullptr, stage = nullptr, mass = nullptr;
  adj_fn adj_hats = nullptr, adj_mass = nullptr;
  adj_face_fn adj_face = nullptr;
  pack_fn pack = nullptr;
  size_t basis_size = 0;
};

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
    b.ElA[d] = h.ElA[d]; b.E1D[d] = h.E1D[d]; b.E1F[d] = h.E1F[d];
    for (int c = 0; c < NU; ++c) { b.K1[d][c] = h.K1[d][c]; b.Q[d][c] = h.Q[d][c]; b.ilam2[d][c] = h.ilam2[d][c]; }
  }
  for (int r = 0; r < QH; ++r) {
    b.wh[r] = h.wh[r];
    for (int d = 0; d < NV; ++d) { b.Ph[r][d] = h.Ph[r][d]; b.PhW[r][d] = h.PhW[r][d]; }
  }
}

template <int NU, int NV>
void launch_prep(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads, cudaStream_t st) {
  k_prep<NU, NV><<<blocks, threads, 0, st>>>(*static_cast<const Basis<NU, NV> *>(basis), F, S);
}

// k_stage keeps the element blocks in dynamic shared memory (up to 227 KB per block);
// `threads` must be stage_threads(NU, NV, FAST)
template <int NU, int NV, bool FAST>
void launch_stage(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads, cudaStream_t st) {
  constexpr size_t smem = stage_smem(NU, NV, FAST);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_stage<NU, NV, FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  if (blocks <= 0) return;
  k_stage<NU, NV, FAST><<<blocks, threads, smem, st>>>(*static_cast<const Basis<NU, NV> *>(basis), F, S);
}

// The mass solve: k_cheb or k_cg, a team of threads per element (static shared memory sized
// for CHEB_THREADS). `threads` (32, 64, 96 or 128) sets the warps of a block and with them its
// elements; the grid follows from F.E, `blocks` only says whether to launch.
template <int NU, int NV>
void launch_mass(const void *basis, const Fields &F, const StageIO &S, int blocks, int threads, cudaStream_t st) {
  if (blocks <= 0) return;
  const Basis<NU, NV> &B = *static_cast<const Basis<NU, NV> *>(basis);
  threads = (threads >= 32 && threads <= CHEB_THREADS && threads % 32 == 0) ? threads : CHEB_THREADS;
  const int tpb = (threads / 32) * ChebTeam<NU, NV>::TPW;
  const int grid = (F.E + tpb - 1) / tpb;
  if (F.cg) k_cg<NU, NV><<<grid, threads, 0, st>>>(B, F, S);
  else k_cheb<NU, NV><<<grid, threads, 0, st>>>(B, F, S);
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
Launchers make_launchers(bool fast) {
  Launchers L;
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
