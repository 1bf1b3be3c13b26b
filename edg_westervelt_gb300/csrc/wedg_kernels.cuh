// Device kernels of libwedg: one RHS stage of the EDG scheme for the
// Westervelt equation on sm_103a, FP64.
//
// Design (GB300): the path is bound by the FP64 pipe (about 1.2 TFLOP/s on
// GB300, 1/58 of FP32), not by HBM. The kernels therefore minimise FP64
// instructions and keep all 32 lanes of a warp busy: one thread owns one
// element, with compile-time sizes. The element's modal blocks live in shared
// memory in a [index][thread] layout (conflict-free, and a shared load costs a
// fraction of one 64-cycle FP64 warp instruction), small temporaries in
// registers. Memory is spent freely where it saves arithmetic: traces and
// Chebyshev weights are computed once per stage and re-read.
//
// One RHS evaluation is three kernels:
//   k_prep   traces of the stage state on the four sides of every element
//            (src/rhs.jl:384-410), the weight check of the boundary points
//            (src/rhs.jl:105-110, 729-757) and the Chebyshev interval data
//            (src/rhs.jl:889-907), so that every error of the stage is known
//            before the second kernel starts;
//   k_stage  face fluxes of the element's own sides (src/rhs.jl:611-700,
//            65-103), lifts (:412-473), volume terms (:309-333), source
//            (:335-350) and u-equation (:352-382) with the u part of the RK4
//            stage update (src/solver.jl:299-321); it leaves the right-hand
//            side of the mass system in HBM;
//   k_cheb   the Chebyshev mass solve (:920-939) and the v part of the RK4
//            update, a team of threads per element. Elements are visited in
//            decreasing order of their Chebyshev step counts (k_prep lists them
//            by count), so the longest solves start first;
//   k_cg     the same with conjugate gradients (:821-853), also a team per element.
// Interior faces are evaluated by both neighbours, each writing only its own
// slots, so no element writes another element's data.
//
// Device layouts (element index e = j + N k fastest everywhere):
//   state       x[e + E (a + n b)]                 (the reference's own layout)
//   traces      tr[((fam*4 + side)*NQ + i)*E + e]  fam du, v, dv; side B, T, L, R
//   Cw, Aw      [(r + NQ s) E + e]
//   Ainv        [row E + e]                        packed upper triangle by columns
//   h-faces     [jf + (N+1)(k + N i)]              face row jf, column k, point i
//   v-faces     [j + N (kf + (N+1) i)]
//   bnd data    [m + N i]
//   Pi, srcP    [(a + NV b) E + e]
//   2β, G       [(r + QH s) E + e]
//   mass rhs    [(a + NV b) E + e]
#pragma once
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

namespace wedg {

constexpr unsigned long long ERR_NONE = ~0ull;
constexpr int ERR_CLASS_SHIFT = 56;   // class 0: boundary weight, 1: mass matrix not PD, 3: stopped (non-finite)
constexpr int NBIN = 48;              // Chebyshev-count bins of the mass kernel (the last holds n ≥ NBIN)
constexpr int CHEB_THREADS = 128;    // threads per block of the mass-solve kernels

__host__ __device__ constexpr int qhigh(int nu, int nv) {
  // q_high = max(ceil(3 q_v / 2) + 1, q_u + 1), src/solver.jl:483
  return ((3 * (nv - 1) + 1) / 2 + 1) > nu ? ((3 * (nv - 1) + 1) / 2 + 1) : nu;
}

// Shared memory of k_stage per thread: b and R_v (NU² + NV² doubles); the general kernels give
// R_v NU² doubles, because the packed-inverse u-solve writes its result there once R_v is spent.
// Both read U and V from HBM.
__host__ __device__ constexpr int stage_doubles(int nu, int nv, bool fast) {
  return fast ? nu * nu + nv * nv : 2 * nu * nu;
}
// Threads per block of k_stage: two blocks per SM (228 KB per SM, 1 KB of it per block reserved)
__host__ __device__ constexpr int stage_threads(int nu, int nv, bool fast) {
  return 2 * (128 * stage_doubles(nu, nv, fast) * 8 + 1024) <= 233472 ? 128 : 96;
}
__host__ __device__ constexpr size_t stage_smem(int nu, int nv, bool fast) {
  return (size_t)stage_threads(nu, nv, fast) * stage_doubles(nu, nv, fast) * sizeof(double);
}

template <int NU, int NV>
struct Basis {
  static constexpr int NQ = NU;
  static constexpr int QH = qhigh(NU, NV);
  double w[NQ];
  double P[NQ][NU], S[NQ][NU];   // P[i][d] = P_u[i, d], S likewise; the v-basis is d < NV
  double Pw[NQ][NU];             // w[i] P[i][d]
  double El[NU], Er[NU], E1l[NU], E1r[NU];
  double E1F[NU];                // -E1l, the lift factor of the u-slots (the v-slots' factors
                                 // (2/h) El and (4/h²) E1l take the mesh size from Fields)
  double Ph[QH][NV];             // P_h_v[r, d]
  double PhW[QH][NV];            // w_h[r] P_h_v[r, d], with W2d_h = w_h w_h^T
  double wh[QH];                 // w_h
  double K1[NU][NU];             // 1D stiffness S^T diag(w) S
  double Q[NU][NU];              // its eigenvectors, Q[row][col]; Q[.][0] = e_0
  double ilam2[NU][NU];          // 1 / (λ_i + λ_j), and 1 at (0, 0)
  double QE[NU];                 // Q^T E1F: the u-slots' lift factor in the eigenbasis of K1
};

struct Fields {
  int N, E;
  const double *Cw, *Aw, *Ainv, *ic2e, *c2e, *ae;
  const double *hc2, *haf, *hcf, *hbf, *hc2m, *hafm, *hJC;
  const double *vc2, *vaf, *vcf, *vbf, *vc2m, *vafm, *vJC;
  // with modal traces and one-sided faces: the jump terms' projections Σ_i w_i P[i][b] JC_i on the
  // face modes b, in the layouts of hJC, vJC with mode b in the slot of point b (null: no jump term)
  const double *hJCm, *vJCm;
  const double *bsp[4], *bspn[4];
  const double *PiSP, *PiBSP2, *PiCdiv, *PiDdiv, *srcP;
  const double *beta2;        // 2β at the high-order points, [(r + QH s) E + e]
  double *tr, *G, *th, *de;   // G = 2βv at the high-order points
  double *mrhs;               // right-hand side of the mass system, [(a + NV b) E + e]
  int *nst;
  int *nmax;                  // largest Chebyshev count: [parity] of a stage (the common count of
                              // src/rhs.jl:911-918), [2] of the whole call (statistics)
  int *bins, *bin_count;      // elements by Chebyshev count: bins[b E + i], two count buffers of NBIN
  unsigned long long *nsum;   // Σ of the per-element Chebyshev step counts
  unsigned long long *err;
  unsigned int *cg_nfail, *nonfinite;
  double theta, tau, lu, lv, omega, two_h, four_hh, mass_tol, Lcheb;
  int one_sided, mms_on, src_on, cg, cheb_common, sorted;
  // modal traces: tr holds each side's modal end sums (index b < n in place of point i), and the
  // interior slots are projected in that form (every interior face's coefficients are one value
  // along the face; the adjoint kernels read point traces)
  int modal;
  int kind[4];
  double gam[4], eta[4], sig[4], kb[4], kap[4];
};

enum StageMode {
  OUT_RHS = 0, OUT_RK4_STAGE = 1, OUT_RK4_LAST = 2, OUT_RK4_LAST_ACC = 3,
  // adjoint parts of k_stage (both forms are symmetric, so the forward code is its own transpose):
  OUT_ADJ_USOLVE = 4,   // ut = A_e⁻¹ xu (the u-solve alone)
  OUT_ADJ_VOLUME = 5    // vt = R_v, ut = b of the volume terms alone, for the state (xu, xv)
};

struct StageIO {
  const double *xu, *xv;     // stage state
  double ct, st, srct;       // time factors of the stage (src/rhs.jl:509-511)
  double cSP, cB, cC, cD;    // source weights: -ω²ct, -2ω³ st ct, 1 - ct, ω st
  // or, for launches replayed from a CUDA graph, the same seven factors (and one pad) from a
  // host-computed table of tf_n steps: tf[((step mod tf_n)·4 + stage)·8 + f], step = *step (the
  // workspace's device step counter); the host refills the table every tf_n steps
  const double *tf;
  const long long *step;
  long long tf_n;
  int stage;
  int mode, first;
  int parity;                // which bin-count buffer this stage fills (the other is cleared)
  double *ut, *vt;           // OUT_RHS
  const double *u0, *v0;     // RK4 base state
  double *su, *sv;           // next stage state
  double *accu, *accv;       // k1 + 2k2 + 2k3 (+ k4)
  double *uo, *vo;           // in-place target of the last stage
  double c;                  // next-stage factor, or dt/6 on the last stage
};

// The time factors of a stage: from the launch parameters, or from the table of a graph replay
struct TimeF {
  double ct, st, srct, cSP, cB, cC, cD;
};
__device__ __forceinline__ TimeF time_factors(const StageIO &S) {
  if (!S.tf) return TimeF{S.ct, S.st, S.srct, S.cSP, S.cB, S.cC, S.cD};
  long long it = *(volatile const long long *)S.step;
  it = it < 0 ? 0 : it % S.tf_n;
  const double *f = S.tf + (it * 4 + S.stage) * 8;
  return TimeF{f[0], f[1], f[2], f[3], f[4], f[5], f[6]};
}

__device__ __forceinline__ unsigned long long err_word(const Fields &F) {
  return *(volatile unsigned long long *)F.err;
}

// ----------------------------------------------------------------------------
// Multi-instance launches (the batched form): one launch runs one kernel of a stage for up to
// CAP instances with the same degrees (so the same kernel and the same 1D operators) and
// any mesh sizes. Their arguments travel in the launch's parameter block. The launch covers
// first[n] virtual blocks: virtual block vb belongs to the instance i with first[i] ≤ vb <
// first[i+1] and covers `tile` elements (or element slots of the mass solves' order) of it,
// from (vb - first[i]) tile on. Each block copies its instance's arguments into shared memory
// and runs the single-instance kernel's body on them, so an element's arithmetic is the same
// as in a launch of its instance alone. A grid smaller than first[n] makes the launch
// persistent: block b takes the virtual blocks b, b + gridDim.x, ...
// ----------------------------------------------------------------------------
struct StageArgs {
  Fields F;
  StageIO S;
};

template <class Args, int CAP>
struct Multi {
  static constexpr int cap = CAP;
  int n, tile;
  int first[CAP + 1];
  Args a[CAP];
};

// CAP is what fits the kernel parameter limit (32 764 bytes) beside the largest Basis
using MultiStage = Multi<StageArgs, 31>;

// The instance of virtual block vb. The kernels read that instance's arguments where they lie, in
// the parameter block: the index is the same for the whole block, so the reads are uniform
// constant-bank loads. The barrier keeps a persistent block's next virtual block from reusing
// shared memory that threads of the previous one still read.
template <class Args, int CAP>
__device__ __forceinline__ int multi_begin(const Multi<Args, CAP> &P, int vb) {
  int inst = 0;
  while (inst + 1 < P.n && vb >= P.first[inst + 1]) ++inst;
  __syncthreads();
  return inst;
}

// A thread-private n×n block in shared memory: X(a, b) at base[(a + n b) BT + tid]
template <int n, int BT>
struct Blk {
  double *p;
  __device__ __forceinline__ double &operator()(int a, int b) const { return p[(a + n * b) * BT]; }
};

// Nonzero pattern of the eigenbasis Q of the 1D stiffness K1 (built so on the host): Q[a][i]
// vanishes for a + i odd and in row and column 0 outside (0, 0)
__host__ __device__ constexpr bool qnz(int a, int i) { return ((a + i) & 1) == 0 && ((a == 0) == (i == 0)); }

// ----------------------------------------------------------------------------
// Mirror-parity contractions. The points of both quadratures are Gauss-Legendre
// points (mirrored through the element centre) and the basis is the Legendre one,
// so P[n-1-i][d] = (-1)^d P[i][d] for the values and the opposite sign for the
// derivatives (the host makes these exact). A contraction over the modes is then
// done on the first half of the points only -- its even-mode and odd-mode parts give
// the point and its mirror as a sum and a difference -- and a contraction over the
// points from the sums (even modes) and differences (odd modes) of mirrored points.
// ----------------------------------------------------------------------------

// Y[s] = Σ_b T[b] Ph[s][b] at all QH points
template <int QH, int NV>
__device__ __forceinline__ void ph_to_points(const double (&Ph)[QH][NV], const double (&T)[NV], double (&Y)[QH]) {
#pragma unroll
  for (int s = 0; s < QH / 2; ++s) {
    double ev = 0.0, od = 0.0;
#pragma unroll
    for (int b = 0; b < NV; b += 2) ev = fma(T[b], Ph[s][b], ev);
#pragma unroll
    for (int b = 1; b < NV; b += 2) od = fma(T[b], Ph[s][b], od);
    Y[s] = ev + od;
    Y[QH - 1 - s] = ev - od;
  }
  if constexpr ((QH & 1) != 0) {
    double ev = 0.0;
#pragma unroll
    for (int b = 0; b < NV; b += 2) ev = fma(T[b], Ph[QH / 2][b], ev);
    Y[QH / 2] = ev;
  }
}

// Z[b] = Σ_s Y[s] Ph[s][b]
template <int QH, int NV>
__device__ __forceinline__ void ph_from_points(const double (&Ph)[QH][NV], const double (&Y)[QH], double (&Z)[NV]) {
  double ys[QH / 2 + 1], yd[QH / 2 + 1];
#pragma unroll
  for (int s = 0; s < QH / 2; ++s) {
    ys[s] = Y[s] + Y[QH - 1 - s];
    yd[s] = Y[s] - Y[QH - 1 - s];
  }
#pragma unroll
  for (int b = 0; b < NV; ++b) {
    double z = 0.0;
#pragma unroll
    for (int s = 0; s < QH / 2; ++s) z = fma((b & 1) ? yd[s] : ys[s], Ph[s][b], z);
    if constexpr ((QH & 1) != 0) {
      if (!(b & 1)) z = fma(Y[QH / 2], Ph[QH / 2][b], z);
    }
    Z[b] = z;
  }
}

// Rows r and QH-1-r (r < QH/2) of Ph X for an NV×NV block x(a, b):
//   Tp[b] = Σ_a Ph[r][a] x(a, b),  Tm[b] = Σ_a (-1)^a Ph[r][a] x(a, b)
template <int QH, int NV, class X>
__device__ __forceinline__ void ph_row_pair(const double (&Ph)[QH][NV], int r, const X &x, double (&Tp)[NV],
                                            double (&Tm)[NV]) {
#pragma unroll
  for (int b = 0; b < NV; ++b) {
    double ev = 0.0, od = 0.0;
#pragma unroll
    for (int a = 0; a < NV; a += 2) ev = fma(Ph[r][a], x(a, b), ev);
#pragma unroll
    for (int a = 1; a < NV; a += 2) od = fma(Ph[r][a], x(a, b), od);
    Tp[b] = ev + od;
    Tm[b] = ev - od;
  }
}

// The middle row QH/2 of Ph X when QH is odd (only the even modes are nonzero there)
template <int QH, int NV, class X>
__device__ __forceinline__ void ph_row_mid(const double (&Ph)[QH][NV], const X &x, double (&T)[NV]) {
#pragma unroll
  for (int b = 0; b < NV; ++b) {
    double ev = 0.0;
#pragma unroll
    for (int a = 0; a < NV; a += 2) ev = fma(Ph[QH / 2][a], x(a, b), ev);
    T[b] = ev;
  }
}

// ----------------------------------------------------------------------------
// k_prep: traces, boundary weight check, Chebyshev interval data
// ----------------------------------------------------------------------------

// Traces of an n×n block X on the four sides (src/rhs.jl:388-410):
//   oB[i] = Σ_b P[i,b] Σ_a El[a] X[a][b],  oT with Er,
//   oL[i] = Σ_b P[i,b] Σ_a El[a] X[b][a],  oR with Er,
// where El, Er are the values (DER false) or the derivatives (DER true) of the modes at the
// two ends: Er[a] = ±(-1)^a El[a], so both ends come from the even and odd parts of one sum.
// The bottom/top pair (AXIS 0) and the left/right pair (AXIS 1) are separate passes, so that
// only one pair's end sums are live at a time. With SCALE, every output is multiplied by sc.
template <int NQ, int NU, int n, bool DER, int AXIS, bool SCALE>
__device__ __forceinline__ void trace2(const double (&X)[n][n], const double (&P)[NQ][NU], const double *El,
                                       double *tr, int fam, int E, int e, double sc, bool modal) {
  double sA[n], sZ[n];   // the end sums at the low (B or L) and the high (T or R) end
#pragma unroll
  for (int b = 0; b < n; ++b) {
    double xe = 0, xo = 0;
#pragma unroll
    for (int a = 0; a < n; a += 2) xe = fma(El[a], AXIS == 0 ? X[a][b] : X[b][a], xe);
#pragma unroll
    for (int a = 1; a < n; a += 2) xo = fma(El[a], AXIS == 0 ? X[a][b] : X[b][a], xo);
    sA[b] = xe + xo;
    sZ[b] = DER ? xo - xe : xe - xo;
  }
  auto put = [&](int i, double oA, double oZ) {
    if constexpr (SCALE) { oA *= sc; oZ *= sc; }
    tr[((fam * 4 + 2 * AXIS) * NQ + i) * (size_t)E + e] = oA;
    tr[((fam * 4 + 2 * AXIS + 1) * NQ + i) * (size_t)E + e] = oZ;
  };
  if (modal) {            // the end sums themselves, mode b in the slot of point b
#pragma unroll
    for (int b = 0; b < n; ++b) put(b, sA[b], sZ[b]);
    return;
  }
#pragma unroll
  for (int i = 0; i < (NQ + 1) / 2; ++i) {
    double eA = 0, eZ = 0, oA = 0, oZ = 0;
#pragma unroll
    for (int b = 0; b < n; b += 2) { eA = fma(P[i][b], sA[b], eA); eZ = fma(P[i][b], sZ[b], eZ); }
    if (2 * i + 1 == NQ) {      // the middle point: the odd modes vanish there
      put(i, eA, eZ);
      continue;
    }
#pragma unroll
    for (int b = 1; b < n; b += 2) { oA = fma(P[i][b], sA[b], oA); oZ = fma(P[i][b], sZ[b], oZ); }
    put(i, eA + oA, eZ + oZ);
    put(NQ - 1 - i, eA - oA, eZ - oZ);
  }
}

template <int NQ, int NU, int n, bool DER, bool SCALE = false>
__device__ __forceinline__ void trace4(const double (&X)[n][n], const double (&P)[NQ][NU], const double *El,
                                       double *tr, int fam, int E, int e, double sc = 1.0, bool modal = false) {
  trace2<NQ, NU, n, DER, 0, SCALE>(X, P, El, tr, fam, E, e, sc, modal);
  trace2<NQ, NU, n, DER, 1, SCALE>(X, P, El, tr, fam, E, e, sc, modal);
}

// The value at face point i of side `side` of trace family fam of element e held as modal end sums
// (Fields::modal): Σ_b P[i][b] t[b] over the family's n modes
template <int NQ, int NU, int n>
__device__ __forceinline__ double modal_at(const double (&P)[NQ][NU], const double *tr, int fam, int side, int i,
                                           size_t E, int e) {
  double x = 0.0;
#pragma unroll
  for (int b = 0; b < n; ++b) x = fma(P[i][b], tr[((fam * 4 + side) * NQ + b) * E + e], x);
  return x;
}

template <int n>
__device__ __forceinline__ void load_regs(double (&X)[n][n], const double *x, int E, int e) {
#pragma unroll
  for (int b = 0; b < n; ++b)
#pragma unroll
    for (int a = 0; a < n; ++a) X[a][b] = x[e + (size_t)E * (a + n * b)];
}

// k_prep's work for element e (first: the instance's first block, which clears the bin counts)
template <int NU, int NV>
__device__ __forceinline__ void prep_body(const Basis<NU, NV> &B, const Fields &F, const StageIO &S, int e,
                                          bool first) {
  constexpr int NQ = NU, QH = Basis<NU, NV>::QH;
  const int E = F.E, N = F.N;
  // the bin counts and the largest count of the next stage start at zero: all NBIN bins, whatever
  // the element count
  if (first && F.sorted)
    for (int b = threadIdx.x; b < NBIN; b += blockDim.x) F.bin_count[(1 - S.parity) * NBIN + b] = 0;
  if (first && threadIdx.x == 0) F.nmax[1 - S.parity] = 0;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int j = e % N, k = e / N;
  const bool modal = F.modal != 0;
  {
    double U[NU][NU];
    load_regs<NU>(U, S.xu, E, e);
    trace4<NQ, NU, NU, true>(U, B.P, B.E1l, F.tr, 0, E, e, 1.0, modal);
  }
  double V[NV][NV];
  load_regs<NV>(V, S.xv, E, e);
  trace4<NQ, NU, NV, false>(V, B.P, B.El, F.tr, 1, E, e, 1.0, modal);
  trace4<NQ, NU, NV, true>(V, B.P, B.E1l, F.tr, 2, E, e, 1.0, modal);

  const TimeF tf = time_factors(S);
  // weight check 1 - kβv > 0 for the trace and the data on physical sides
  // (src/rhs.jl:109-110, 751-757); key of src/rhs.jl:732
  const bool onb[4] = {j == 0, j == N - 1, k == 0, k == N - 1};
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    if (!onb[s] || F.kind[s] == 3) continue;
    const int m = s < 2 ? k : j;
    unsigned long long key = ERR_NONE;
#pragma unroll 1
    for (int i = 0; i < NQ; ++i) {
      const double bf = s < 2 ? F.hbf[(s == 0 ? 0 : N) + (size_t)(N + 1) * (k + (size_t)N * i)]
                              : F.vbf[j + (size_t)N * ((s == 2 ? 0 : N) + (size_t)(N + 1) * i)];
      const double v_fp = modal ? modal_at<NQ, NU, NV>(B.P, F.tr, 1, s, i, E, e)
                                : F.tr[((1 * 4 + s) * NQ + i) * (size_t)E + e];
      const double v_ex = -F.omega * tf.st * F.bsp[s][m + (size_t)N * i];
      const int check = (1.0 - F.kb[s] * bf * v_fp <= 0.0) ? 1 : (1.0 - F.kb[s] * bf * v_ex <= 0.0) ? 2 : 0;
      if (check) {
        const unsigned long long kk =
            2ull * ((unsigned long long)s * NQ * N + i + (unsigned long long)m * NQ) + check;
        key = kk < key ? kk : key;
      }
    }
    if (key != ERR_NONE) atomicMin(F.err, key);
  }

  if (F.cg) return;
  // Chebyshev interval of the element: v_q = P_h V P_h^T, G = 2βv_q, a± = 1 - extrema(G);
  // the rows of the point grid in mirrored pairs. The extrema and the NaN test run on the
  // integer pipe (order-preserving integer keys of the doubles), so that a point costs one
  // FP64 multiply besides the contractions.
  long long kmin = LLONG_MAX, kmax = LLONG_MIN;
  bool nan = false;
  auto vx = [&](int a, int b) { return V[a][b]; };
  auto point = [&](double y, int r, int s2) {
    const size_t gi = (r + QH * s2) * (size_t)E + e;
    const double g = y * F.beta2[gi];
    F.G[gi] = g;
    const long long bits = __double_as_longlong(g);
    nan |= (bits & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
    const long long key = bits ^ ((bits >> 63) & 0x7fffffffffffffffLL);
    kmin = min(kmin, key);
    kmax = max(kmax, key);
  };
  // the points of row r: v_q = Σ_b T[b] Ph[s2][b], mirrored columns s2 and QH-1-s2 together
  auto points = [&](const double (&T)[NV], int r) {
#pragma unroll
    for (int s2 = 0; s2 < QH / 2; ++s2) {
      double ev = 0.0, od = 0.0;
#pragma unroll
      for (int b = 0; b < NV; b += 2) ev = fma(T[b], B.Ph[s2][b], ev);
#pragma unroll
      for (int b = 1; b < NV; b += 2) od = fma(T[b], B.Ph[s2][b], od);
      point(ev + od, r, s2);
      point(ev - od, r, QH - 1 - s2);
    }
    if constexpr ((QH & 1) != 0) {
      double ev = 0.0;
#pragma unroll
      for (int b = 0; b < NV; b += 2) ev = fma(T[b], B.Ph[QH / 2][b], ev);
      point(ev, r, QH / 2);
    }
  };
#pragma unroll 1
  for (int r = 0; r < QH / 2; ++r) {
    double Tp[NV], Tm[NV];
    ph_row_pair<QH, NV>(B.Ph, r, vx, Tp, Tm);
    points(Tp, r);
    points(Tm, QH - 1 - r);
  }
  if constexpr ((QH & 1) != 0) {
    double T[NV];
    ph_row_mid<QH, NV>(B.Ph, vx, T);
    points(T, QH / 2);
  }
  const double gmin = __longlong_as_double(kmin ^ ((kmin >> 63) & 0x7fffffffffffffffLL));
  const double gmax = __longlong_as_double(kmax ^ ((kmax >> 63) & 0x7fffffffffffffffLL));
  const double amin = 1.0 - gmax, amax = 1.0 - gmin;
  if (nan || !(amin > 0.0)) {
    atomicMin(F.err, (1ull << ERR_CLASS_SHIFT) | (unsigned long long)(e + 1));
    return;
  }
  const double th = 0.5 * (amax + amin);
  const double de = fmax(0.5 * (amax - amin), 1e-15 * th);
  F.th[e] = th;
  F.de[e] = de;
  const int n = (int)ceil(F.Lcheb / acosh(th / de));
  F.nst[e] = n;
  // largest count and the sum of the counts: one atomic each per warp
  const unsigned mask = __activemask();
  const int nw = __reduce_max_sync(mask, n);
  const unsigned ns = __reduce_add_sync(mask, (unsigned)n);
  const int lane = threadIdx.x & 31;
  if (lane == __ffs(mask) - 1) {
    atomicMax(&F.nmax[S.parity], nw);
    atomicMax(&F.nmax[2], nw);
    atomicAdd(F.nsum, (unsigned long long)ns);
  }
  if (F.sorted) {
    // append e to the list of its count, one atomic per group of lanes with the same count
    const int bin = (n < NBIN ? n : NBIN) - 1;
    const unsigned same = __match_any_sync(mask, bin);
    const int leader = __ffs(same) - 1;
    const int rank = __popc(same & ((1u << lane) - 1));
    int base = 0;
    if (lane == leader) base = atomicAdd(&F.bin_count[S.parity * NBIN + bin], __popc(same));
    base = __shfl_sync(same, base, leader);
    F.bins[(size_t)bin * E + base + rank] = e;
  }
}

template <int NU, int NV>
__global__ void __launch_bounds__(128, 3) k_prep(const __grid_constant__ Basis<NU, NV> B,
                                              const __grid_constant__ Fields F,
                                              const __grid_constant__ StageIO S, int e0) {
  // elements e0 + (block, thread): a launch may cover a range of the elements (the first range
  // clears the next stage's counts)
  prep_body<NU, NV>(B, F, S, e0 + (int)(blockIdx.x * blockDim.x + threadIdx.x), blockIdx.x == 0 && e0 == 0);
}

template <int NU, int NV>
__global__ void __launch_bounds__(128, 3) k_prep_m(const __grid_constant__ Basis<NU, NV> B,
                                                const __grid_constant__ MultiStage P) {
  for (int vb = blockIdx.x; vb < P.first[P.n]; vb += gridDim.x) {
    const int inst = multi_begin(P, vb);
    const int e0 = (vb - P.first[inst]) * P.tile;
    prep_body<NU, NV>(B, P.a[inst].F, P.a[inst].S, e0 + (int)threadIdx.x, e0 == 0);
  }
}

// ----------------------------------------------------------------------------
// k_stage helpers
// ----------------------------------------------------------------------------

// Coefficients of an interior face point: the one-sided values of c² and α on the "-" and "+"
// sides and the jump term K (one-sided faces), or the face values c², α (continuous faces)
struct FaceCoef {
  double c2m, c2p, afm, afp, K;
};
__device__ __forceinline__ FaceCoef face_coef(const Fields &F, const double *c2p_a, const double *afp_a,
                                              const double *c2m_a, const double *afm_a, const double *jc_a,
                                              size_t fi) {
  if (F.one_sided) return FaceCoef{c2m_a[fi], c2p_a[fi], afm_a[fi], afp_a[fi], jc_a[fi]};
  return FaceCoef{0.0, c2p_a[fi], 0.0, afp_a[fi], 0.0};
}

// The flux slots of the "+" (plus) or "-" element at an interior face point from the traces of
// both elements (src/rhs.jl:620-700): affine in (dum, dup, vm, vp, dvm, dvp)
__device__ __forceinline__ void interior_flux(const Fields &F, const FaceCoef &cf, bool plus, double dum,
                                              double dup, double vm, double vp, double dvm, double dvp,
                                              double &A, double &D, double &Fs) {
  const double th = F.theta, tau = F.tau, two_h = F.two_h;
  if (F.one_sided) {
    const double c2m = cf.c2m, c2p = cf.c2p, afm = cf.afm, afp = cf.afp, K = cf.K;
    const double J = two_h * (c2m * dum - c2p * dup + afm * dvm - afp * dvp) + K;
    const double G = two_h * ((1 - th) * (c2m * dum + afm * dvm) + th * (c2p * dup + afp * dvp));
    const double pen = (0.5 * (c2m + c2p)) * F.lu + (0.5 * (afm + afp)) * F.lv;
    const double sj = vm - vp;
    if (plus) {
      const double dvsp = th * sj - tau * J;
      A = pen * sj - G - (1 - th) * K; D = -afp * dvsp; Fs = c2p * dvsp;
    } else {
      const double dvsm = (1 - th) * (vp - vm) - tau * J;
      A = G - pen * sj - th * K; D = afm * dvsm; Fs = -c2m * dvsm;
    }
  } else {
    const double c2 = cf.c2p, af = cf.afp;
    const double gs = two_h * (c2 * (th * dup + (1 - th) * dum) + af * (th * dvp + (1 - th) * dvm));
    const double Jt = c2 * (two_h * (dum - dup)) + af * (two_h * (dvm - dvp));
    const double pen = c2 * F.lu + af * F.lv;
    if (plus) {
      A = pen * (vm - vp) - gs;
      D = -af * (th * (vm - vp) - tau * Jt);
      Fs = c2 * (th * (vm - vp) - tau * Jt);
    } else {
      A = gs - pen * (vm - vp);
      D = af * ((1 - th) * (vp - vm) - tau * Jt);
      Fs = -c2 * ((1 - th) * (vp - vm) - tau * Jt);
    }
  }
}

// Numerical flux slots A, D, F at point i of side s of the element
// (src/rhs.jl:620-700 for interior faces, :65-103 and :738-763 for physical sides).
template <int NU, int NV>
__device__ __forceinline__ void side_point(const Basis<NU, NV> &B, const Fields &F, const TimeF &S, int s,
                                           bool boundary, int j, int k, int e, int i, double &A, double &D,
                                           double &Fs) {
  constexpr int NQ = NU;
  const int N = F.N, E = F.E;
  const double *tr = F.tr;
  auto T = [&](int fam, int side, int el) { return tr[((fam * 4 + side) * NQ + i) * (size_t)E + el]; };
  if (boundary) {
    const int m = s < 2 ? k : j;
    const double sgn = (s == 0 || s == 2) ? -1.0 : 1.0;
    size_t fi;
    const double *c2a, *afa, *cfa, *bfa;
    if (s < 2) { fi = (s == 0 ? 0 : N) + (size_t)(N + 1) * (k + (size_t)N * i); c2a = F.hc2; afa = F.haf; cfa = F.hcf; bfa = F.hbf; }
    else { fi = j + (size_t)N * ((s == 2 ? 0 : N) + (size_t)(N + 1) * i); c2a = F.vc2; afa = F.vaf; cfa = F.vcf; bfa = F.vbf; }
    const double c2f = c2a[fi], af = afa[fi], cf = cfa[fi];
    const bool modal = F.modal != 0;
    const double v_fp = modal ? modal_at<NQ, NU, NV>(B.P, tr, 1, s, i, E, e) : T(1, s, e);
    const double gun = sgn * (F.two_h * (modal ? modal_at<NQ, NU, NU>(B.P, tr, 0, s, i, E, e) : T(0, s, e)));
    const double gvn = sgn * (F.two_h * (modal ? modal_at<NQ, NU, NV>(B.P, tr, 2, s, i, E, e) : T(2, s, e)));
    const double spn = F.bspn[s][m + (size_t)N * i], sp = F.bsp[s][m + (size_t)N * i];
    const double gu_ex = sgn * (S.ct * spn - spn);
    const double gv_ex = sgn * (-F.omega * S.st * spn);
    const double v_ex = -F.omega * S.st * sp;
    double F1, dv;
    if (F.kind[s] == 3) {
      const double g2 = c2f * gu_ex + af * gv_ex;
      const double rho_w = c2f * gun + af * gvn - g2;
      dv = -(F.kap[s] / cf) * rho_w;
      F1 = g2;
    } else {
      const double bf = bfa[fi];
      const double g = F.gam[s], et = F.eta[s], sg = F.sig[s], kb = F.kb[s];
      const double sqf = sqrt(1.0 - kb * bf * v_fp);
      const double rho_num = et * (c2f * gun + af * gvn) + g * cf * sqf * v_fp;
      const double rho_ex = et * (c2f * gu_ex + af * gv_ex) + g * cf * sqrt(1.0 - kb * bf * v_ex) * v_ex;
      const double rho = rho_num - rho_ex;
      F1 = c2f * gun + af * gvn - (et + sg * g) * rho;
      dv = -(g - sg * et) / (cf * sqf) * rho;
    }
    A = F1;
    D = sgn * (af * dv);
    Fs = -sgn * (c2f * dv);
    return;
  }
  // interior: the element is "+" on its B and L sides, "-" on T and R
  const bool plus = (s == 0 || s == 2);
  const int nb = s == 0 ? e - 1 : s == 1 ? e + 1 : s == 2 ? e - N : e + N;
  const int sm = s < 2 ? 1 : 3, spp = s < 2 ? 0 : 2;      // trace sides of the "-" and "+" elements
  const int em = plus ? nb : e, ep = plus ? e : nb;
  size_t fi;
  const double *c2p_a, *afp_a, *c2m_a, *afm_a, *jc_a;
  if (s < 2) {
    fi = (s == 0 ? j : j + 1) + (size_t)(N + 1) * (k + (size_t)N * i);
    c2p_a = F.hc2; afp_a = F.haf; c2m_a = F.hc2m; afm_a = F.hafm; jc_a = F.hJC;
  } else {
    fi = j + (size_t)N * ((s == 2 ? k : k + 1) + (size_t)(N + 1) * i);
    c2p_a = F.vc2; afp_a = F.vaf; c2m_a = F.vc2m; afm_a = F.vafm; jc_a = F.vJC;
  }
  const double vm = T(1, sm, em), vp = T(1, spp, ep);
  const double dum = T(0, sm, em), dup = T(0, spp, ep);
  const double dvm = T(2, sm, em), dvp = T(2, spp, ep);
  const FaceCoef cf = face_coef(F, c2p_a, afp_a, c2m_a, afm_a, jc_a, fi);
  interior_flux(F, cf, plus, dum, dup, vm, vp, dvm, dvp, A, D, Fs);
}

// The projections Y_A, Y_D (b < NV) and Y_F (b < NU) of the flux slots of interior side s, with
// the traces held as modal end sums (Fields::modal). The face coefficients are one value along the
// face, so every slot is a linear combination of the six traces and the jump term K with the same
// weights at every point, and its projection Σ_i w_i P[i][b] (.)_i is that combination of the
// traces' modes b and of K's projection on mode b (hJCm, vJCm): the face rule integrates the
// product of two modes exactly and the modes are orthonormal. The same results as the point form
// of side_point and the projections, to rounding.
template <int NU, int NV>
__device__ __forceinline__ void modal_side(const Fields &F, int s, int j, int k, int e, double (&YA)[NV],
                                           double (&YD)[NV], double (&YF)[NU]) {
  constexpr int NQ = NU;
  const int N = F.N;
  const size_t E = F.E;
  const bool plus = (s == 0 || s == 2);
  const int nb = s == 0 ? e - 1 : s == 1 ? e + 1 : s == 2 ? e - N : e + N;
  const int sm = s < 2 ? 1 : 3, spp = s < 2 ? 0 : 2;      // trace sides of the "-" and "+" elements
  const int em = plus ? nb : e, ep = plus ? e : nb;
  size_t fi;
  const double *c2p_a, *afp_a, *c2m_a, *afm_a, *jc_a, *jcm;
  if (s < 2) {
    fi = (s == 0 ? j : j + 1) + (size_t)(N + 1) * k;
    c2p_a = F.hc2; afp_a = F.haf; c2m_a = F.hc2m; afm_a = F.hafm; jc_a = F.hJC; jcm = F.hJCm;
  } else {
    fi = j + (size_t)N * (s == 2 ? k : k + 1);
    c2p_a = F.vc2; afp_a = F.vaf; c2m_a = F.vc2m; afm_a = F.vafm; jc_a = F.vJC; jcm = F.vJCm;
  }
  const FaceCoef cf = face_coef(F, c2p_a, afp_a, c2m_a, afm_a, jc_a, fi);   // point 0 of the face
  // the slots of interior_flux as linear forms with the face's weights (continuous faces: the
  // one-sided form with equal values on both sides): G = Σ g·traces, J = Σ j·traces + K,
  // s = v⁻ - v⁺; "+": A = pen s - G - (1-θ)K, w = θ s - τJ, D = -α⁺ w, F = c²⁺ w;
  // "-": A = G - pen s - θK, w = -(1-θ) s - τJ, D = α⁻ w, F = -c²⁻ w
  const double th = F.theta, tau = F.tau, two_h = F.two_h;
  const double c2m = F.one_sided ? cf.c2m : cf.c2p, afm = F.one_sided ? cf.afm : cf.afp;
  const double c2p = cf.c2p, afp = cf.afp;
  const double g_um = two_h * ((1 - th) * c2m), g_up = two_h * (th * c2p);
  const double g_vm = two_h * ((1 - th) * afm), g_vp = two_h * (th * afp);
  const double j_um = two_h * c2m, j_up = -(two_h * c2p), j_vm = two_h * afm, j_vp = -(two_h * afp);
  const double pen = (0.5 * (c2m + c2p)) * F.lu + (0.5 * (afm + afp)) * F.lv;
  const double sw = plus ? th : -(1 - th);                 // w = sw s - τJ
  const double kA = plus ? -(1 - th) : -th;                // A = ±(pen s - G) + kA K
  const double dD = plus ? -afp : afm, dF = plus ? c2p : -c2m;
  const size_t fstride = (size_t)(N + 1) * N;              // from point (mode) b to b + 1
  const double *tr = F.tr;
  // mode b of trace family fam on side `side` of element el
  auto T = [&](int fam, int side, int el, int b) { return tr[((fam * 4 + side) * NQ + b) * E + el]; };
#pragma unroll
  for (int b = 0; b < NU; ++b) {
    const double dum = T(0, sm, em, b), dup = T(0, spp, ep, b);
    double G = fma(g_um, dum, g_up * dup), J = fma(j_um, dum, j_up * dup), sj = 0.0;
    if (b < NV) {
      const double vm = T(1, sm, em, b), vp = T(1, spp, ep, b);
      const double dvm = T(2, sm, em, b), dvp = T(2, spp, ep, b);
      G = fma(g_vp, dvp, fma(g_vm, dvm, G));
      J = fma(j_vp, dvp, fma(j_vm, dvm, J));
      sj = vm - vp;
    }
    const double K = jcm ? jcm[fi + fstride * b] : 0.0;
    J += K;
    const double w = fma(sw, sj, -tau * J);
    if (b < NV) {
      const double a = fma(pen, sj, -G);
      YA[b] = fma(kA, K, plus ? a : -a);
      YD[b] = dD * w;
    }
    YF[b] = dF * w;
  }
}

// ----------------------------------------------------------------------------
// k_stage: fluxes, lifts, volume, source, u-equation; the mass right-hand side to HBM
// ----------------------------------------------------------------------------
// k_stage's work for element e, whose blocks live in the shared-memory slot tid of the block
template <int NU, int NV, bool FAST>
__device__ __forceinline__ void stage_body(const Basis<NU, NV> &B, const Fields &F, const StageIO &S, int e,
                                           int tid) {
  constexpr int NQ = NU, BT = stage_threads(NU, NV, FAST);
  extern __shared__ double smem[];
  const int E = F.E, N = F.N;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int j = e % N, k = e / N;
  const double two_h = F.two_h, four_hh = F.four_hh;
  const TimeF tf = time_factors(S);
  // thread-private blocks: b (NU², the u-equation right-hand side, then UT) and R_v (NV², the
  // v-equation right-hand side; in the general kernels its space, NU², then takes UT)
  Blk<NU, BT> bb{smem + tid};
  Blk<NV, BT> Rv{smem + NU * NU * BT + tid};

  // ---- faces and lifts (src/rhs.jl:421-473): Rv (v-equation), b = -Fu (u-equation).
  //      The numerical flux slots A, D, F of a side are projected on the modes, Y[b] =
  //      Σ_i w_i P[i][b] (.)_i, from the sums (even b) and differences (odd b) of mirrored points,
  //      and the two sides of an axis are lifted together: the right-end factors are the
  //      left-end ones times ±(-1)^a, so both sides need one rank-one update per slot.
#pragma unroll 1
  for (int a = 0; a < NV; ++a)
#pragma unroll
    for (int b = 0; b < NV; ++b) Rv(a, b) = 0.0;
#pragma unroll 1
  for (int a = 0; a < NU; ++a)
#pragma unroll
    for (int b = 0; b < NU; ++b) bb(a, b) = S.mode == OUT_ADJ_USOLVE ? S.xu[e + (size_t)E * (a + NU * b)] : 0.0;
  const bool adjoint = S.mode >= OUT_ADJ_USOLVE;
  // the forward modes of the constant-coefficient kernels build the u-equation's right-hand side
  // in the eigenbasis of K1 (the adjoint's volume mode needs the plain basis)
  const bool eig = FAST && !adjoint;
#pragma unroll 1
  for (int ax = 0; ax < 2 && !adjoint; ++ax) {
    double A0[NV], D0[NV], F0[NU];          // the projections of the axis' first side (B or L)
    double YA[NV], YD[NV], YF[NU];
#pragma unroll 1
    for (int t = 0; t < 2; ++t) {
      const int s = 2 * ax + t;
      const bool boundary = (s == 0 && j == 0) || (s == 1 && j == N - 1) || (s == 2 && k == 0) || (s == 3 && k == N - 1);
#pragma unroll
      for (int b = 0; b < NU; ++b) {
        if (b < NV) { YA[b] = 0.0; YD[b] = 0.0; }
        YF[b] = 0.0;
      }
      if (F.modal && !boundary) {
        modal_side<NU, NV>(F, s, j, k, e, YA, YD, YF);
      } else {
#pragma unroll 1
        for (int i = 0; i < NQ / 2; ++i) {
          double A1, D1, F1, A2, D2, F2;
          side_point<NU, NV>(B, F, tf, s, boundary, j, k, e, i, A1, D1, F1);
          side_point<NU, NV>(B, F, tf, s, boundary, j, k, e, NQ - 1 - i, A2, D2, F2);
          const double as = A1 + A2, ad = A1 - A2, ds = D1 + D2, dd = D1 - D2, fs = F1 + F2, fd = F1 - F2;
#pragma unroll
          for (int b = 0; b < NU; ++b) {
            const double p = B.Pw[i][b];
            if (b < NV) {
              YA[b] = fma(p, (b & 1) ? ad : as, YA[b]);
              YD[b] = fma(p, (b & 1) ? dd : ds, YD[b]);
            }
            YF[b] = fma(p, (b & 1) ? fd : fs, YF[b]);
          }
        }
        if constexpr ((NQ & 1) != 0) {         // the middle point: the odd modes vanish there
          double A1, D1, F1;
          side_point<NU, NV>(B, F, tf, s, boundary, j, k, e, NQ / 2, A1, D1, F1);
#pragma unroll
          for (int b = 0; b < NU; b += 2) {
            const double p = B.Pw[NQ / 2][b];
            if (b < NV) {
              YA[b] = fma(p, A1, YA[b]);
              YD[b] = fma(p, D1, YD[b]);
            }
            YF[b] = fma(p, F1, YF[b]);
          }
        }
      }
      if (t == 0) {
#pragma unroll
        for (int b = 0; b < NU; ++b) {
          if (b < NV) { A0[b] = YA[b]; D0[b] = YD[b]; }
          F0[b] = YF[b];
        }
      }
    }
    // lifts of both sides: with σ_a = (-1)^a, El = the left-end values, E1l the left-end
    // derivatives, Rv += El ⊗ (2/h)(A_0 + σ A_1) + E1l ⊗ (4/h²)(D_0 - σ D_1) and
    // b -= E1l ⊗ (F_0 - σ F_1) (B/T: the row index carries E; L/R: the column index)
#pragma unroll
    for (int b = 0; b < NU; ++b) {
      if (b < NV) {
        const double ap = A0[b] + YA[b], am = A0[b] - YA[b], dp = D0[b] + YD[b], dm = D0[b] - YD[b];
        // even-σ and odd-σ combinations, with the mesh factors of the v-slots
        A0[b] = two_h * ap; YA[b] = two_h * am; D0[b] = four_hh * dm; YD[b] = four_hh * dp;
      }
      const double fp = F0[b] + YF[b], fm = F0[b] - YF[b];
      F0[b] = fm; YF[b] = fp;
    }
    if (eig) {
      // the u-slots' lifts straight into the eigenbasis of K1: Q^T (E1F_even ⊗ F_0 + E1F_odd ⊗ F_1) Q
      // = QE_even ⊗ Q^T F_0 + QE_odd ⊗ Q^T F_1 (QE = Q^T E1F keeps the parity of its index)
      double t0[NU], t1[NU];
#pragma unroll
      for (int i = 0; i < NU; ++i) { t0[i] = 0.0; t1[i] = 0.0; }
#pragma unroll
      for (int a = 0; a < NU; ++a)
#pragma unroll
        for (int i = 0; i < NU; ++i)
          if (qnz(a, i)) { t0[i] = fma(B.Q[a][i], F0[a], t0[i]); t1[i] = fma(B.Q[a][i], YF[a], t1[i]); }
#pragma unroll
      for (int i = 0; i < NU; ++i) { F0[i] = t0[i]; YF[i] = t1[i]; }
    }
    const double *LF = eig ? B.QE : B.E1F;
    if (ax == 0) {
#pragma unroll 1
      for (int a = 0; a < NV; ++a) {
        const double ca = B.El[a], cd = B.E1l[a];
        const bool od = a & 1;
#pragma unroll
        for (int b = 0; b < NV; ++b)
          Rv(a, b) = fma(cd, od ? YD[b] : D0[b], fma(ca, od ? YA[b] : A0[b], Rv(a, b)));
      }
#pragma unroll 1
      for (int a = 0; a < NU; ++a) {
        const double ce = LF[a];
        const bool od = a & 1;
#pragma unroll
        for (int b = 0; b < NU; ++b) bb(a, b) = fma(ce, od ? YF[b] : F0[b], bb(a, b));
      }
    } else {
#pragma unroll
      for (int a = 0; a < NV; ++a) {
#pragma unroll
        for (int b = 0; b < NV; ++b)
          Rv(a, b) = fma(B.E1l[b], (b & 1) ? YD[a] : D0[a], fma(B.El[b], (b & 1) ? YA[a] : A0[a], Rv(a, b)));
      }
#pragma unroll
      for (int a = 0; a < NU; ++a) {
#pragma unroll
        for (int b = 0; b < NU; ++b) bb(a, b) = fma(LF[b], (b & 1) ? YF[a] : F0[a], bb(a, b));
      }
    }
  }

  // ---- the state of the stage is read from HBM (by rows of modes in the general kernels, by
  //      columns and by rows in the constant-coefficient kernels)
  const size_t Eu = (size_t)E;
  if (S.mode != OUT_ADJ_USOLVE) {

  // ---- volume terms (src/rhs.jl:309-333): Rv += -4/h² [(c²∇φ_v,∇u_h) + (α∇φ_v,∇v_h)],
  //      b += (c²∇φ_u, ∇v_h)
  if constexpr (FAST) {
    // constant c², α on the element: Cw = c² W, Aw = α W, so that with the
    // 1D stiffness K1 = S^T diag(w) S and the orthonormality of the basis
    //   (c²∇φ_v,∇u_h) + (α∇φ_v,∇v_h) = (K1 W + W K1)[v-block] / (-4/h²),  W = -4/h² (c² U + α V)
    //   (c²∇φ_u, ∇v_h) = c² (K1[:, v] V + V K1[v, :])
    // (V padded with zeros to NU × NU; row and column 0 of K1 vanish, and K1 couples only modes
    // of equal parity). The products with K1 from the left take the columns of U and V, those
    // from the right their rows: both are read from HBM (L2), so that U and V need no shared
    // memory.
    const double c2 = F.c2e[e], al = F.ae[e];
    const double mc2 = -four_hh * c2, mal = -four_hh * al;
    const double *xu = S.xu + e, *xv = S.xv + e;
#pragma unroll 1
    for (int b = 0; b < NV; ++b) {                  // columns: K1 W and K1[:, v] V
      double w[NU], vc[NV];
#pragma unroll
      for (int c = 1; c < NU; ++c) {
        const double uc = xu[Eu * (c + NU * b)];
        if (c < NV) {
          const double x = xv[Eu * (c + NV * b)];
          w[c] = fma(mal, x, mc2 * uc);
          vc[c] = c2 * x;
        } else {
          w[c] = mc2 * uc;
        }
      }
#pragma unroll
      for (int a = 1; a < NU; ++a) {
        if (a < NV) {
          double acc = Rv(a, b);
#pragma unroll
          for (int c = 2 - (a & 1); c < NU; c += 2) acc = fma(B.K1[a][c], w[c], acc);
          Rv(a, b) = acc;
        }
        if (!eig) {
          double acc = bb(a, b);
#pragma unroll
          for (int c = 2 - (a & 1); c < NV; c += 2) acc = fma(B.K1[a][c], vc[c], acc);
          bb(a, b) = acc;
        }
      }
    }
#pragma unroll 1
    for (int a = 0; a < NV; ++a) {                  // rows: W K1 and V K1[v, :]
      double w[NU], vr[NV];
#pragma unroll
      for (int c = 1; c < NU; ++c) {
        const double uc = xu[Eu * (a + NU * c)];
        if (c < NV) {
          const double x = xv[Eu * (a + NV * c)];
          w[c] = fma(mal, x, mc2 * uc);
          vr[c] = c2 * x;
        } else {
          w[c] = mc2 * uc;
        }
      }
#pragma unroll
      for (int b = 1; b < NU; ++b) {
        if (b < NV) {
          double acc = Rv(a, b);
#pragma unroll
          for (int c = 2 - (b & 1); c < NU; c += 2) acc = fma(w[c], B.K1[c][b], acc);
          Rv(a, b) = acc;
        }
        if (!eig) {
          double acc = bb(a, b);
#pragma unroll
          for (int c = 2 - (b & 1); c < NV; c += 2) acc = fma(vr[c], B.K1[c][b], acc);
          bb(a, b) = acc;
        }
      }
    }
  } else {
#pragma unroll 1
    for (int r = 0; r < NQ; ++r) {
      // row r of G1 = S U P^T, G2 = P U S^T and of the same for V
      double tu1[NU], tu2[NU], tv1[NV], tv2[NV];
#pragma unroll
      for (int b = 0; b < NU; ++b) { tu1[b] = 0; tu2[b] = 0; }
#pragma unroll
      for (int b = 0; b < NV; ++b) { tv1[b] = 0; tv2[b] = 0; }
#pragma unroll 1
      for (int a = 0; a < NU; ++a) {
        const double sa = B.S[r][a], pa = B.P[r][a];
#pragma unroll
        for (int b = 0; b < NU; ++b) {
          const double x = S.xu[e + Eu * (a + NU * b)];
          tu1[b] = fma(sa, x, tu1[b]);
          tu2[b] = fma(pa, x, tu2[b]);
        }
        if (a < NV) {
#pragma unroll
          for (int b = 0; b < NV; ++b) {
            const double x = S.xv[e + Eu * (a + NV * b)];
            tv1[b] = fma(sa, x, tv1[b]);
            tv2[b] = fma(pa, x, tv2[b]);
          }
        }
      }
      // the row at the points: g1[s] = Σ_b tu1[b] P[s][b], g2[s] = Σ_b tu2[b] S[s][b], ... from the
      // even and odd modes: P[m][b] = (-1)^b P[s][b] and S[m][b] = -(-1)^b S[s][b] at the mirror
      // point m = NQ-1-s, so the point and its mirror are a sum and a difference
      double g1[NQ], g2[NQ], gv1[NQ], gv2[NQ];
#pragma unroll
      for (int s2 = 0; s2 < (NQ + 1) / 2; ++s2) {
        double pe = 0, po = 0, se = 0, so = 0, qe = 0, qo = 0, te = 0, to = 0;
#pragma unroll
        for (int b = 0; b < NU; ++b) {
          const double pb = B.P[s2][b], sb = B.S[s2][b];
          if (b & 1) {
            po = fma(tu1[b], pb, po); so = fma(tu2[b], sb, so);
            if (b < NV) { qo = fma(tv1[b], pb, qo); to = fma(tv2[b], sb, to); }
          } else {
            pe = fma(tu1[b], pb, pe); se = fma(tu2[b], sb, se);
            if (b < NV) { qe = fma(tv1[b], pb, qe); te = fma(tv2[b], sb, te); }
          }
        }
        g1[s2] = pe + po; g2[s2] = se + so; gv1[s2] = qe + qo; gv2[s2] = te + to;
        if (2 * s2 + 1 != NQ) {
          const int m = NQ - 1 - s2;
          g1[m] = pe - po; g2[m] = so - se; gv1[m] = qe - qo; gv2[m] = to - te;
        }
      }
      // weighted by the coefficients, back to the modes: z1[b] = Σ_s h1[s] P[s][b], ... from the
      // sums and differences of mirrored points
      double h1[NQ], h2[NQ], b1[NQ], b2[NQ];
#pragma unroll
      for (int s2 = 0; s2 < NQ; ++s2) {
        const size_t ci = (r + NQ * s2) * Eu + e;
        const double cw = F.Cw[ci], aw = F.Aw[ci];
        h1[s2] = fma(aw, gv1[s2], cw * g1[s2]);
        h2[s2] = fma(aw, gv2[s2], cw * g2[s2]);
        b1[s2] = cw * gv1[s2];
        b2[s2] = cw * gv2[s2];
      }
      double z1[NV], z2[NV], y1[NU], y2[NU];
#pragma unroll
      for (int b = 0; b < NV; ++b) { z1[b] = 0; z2[b] = 0; }
#pragma unroll
      for (int b = 0; b < NU; ++b) { y1[b] = 0; y2[b] = 0; }
#pragma unroll
      for (int s2 = 0; s2 < (NQ + 1) / 2; ++s2) {
        const bool mid = 2 * s2 + 1 == NQ;
        const int m = NQ - 1 - s2;
        // P-weighted: even modes take the sum, odd the difference; S-weighted: the opposite
        const double h1s = mid ? h1[s2] : h1[s2] + h1[m], h1d = mid ? 0.0 : h1[s2] - h1[m];
        const double h2s = mid ? h2[s2] : h2[s2] + h2[m], h2d = mid ? 0.0 : h2[s2] - h2[m];
        const double b1s = mid ? b1[s2] : b1[s2] + b1[m], b1d = mid ? 0.0 : b1[s2] - b1[m];
        const double b2s = mid ? b2[s2] : b2[s2] + b2[m], b2d = mid ? 0.0 : b2[s2] - b2[m];
#pragma unroll
        for (int b = 0; b < NU; ++b) {
          const double pb = B.P[s2][b], sb = B.S[s2][b];
          const bool odd = b & 1;
          if (b < NV) {
            z1[b] = fma(odd ? h1d : h1s, pb, z1[b]);
            z2[b] = fma(odd ? h2s : h2d, sb, z2[b]);
          }
          y1[b] = fma(odd ? b1d : b1s, pb, y1[b]);
          y2[b] = fma(odd ? b2s : b2d, sb, y2[b]);
        }
      }
#pragma unroll
      for (int b = 0; b < NV; ++b) { z1[b] *= -four_hh; z2[b] *= -four_hh; }
#pragma unroll 1
      for (int a = 0; a < NV; ++a) {
        const double sa = B.S[r][a], pa = B.P[r][a];
#pragma unroll
        for (int b = 0; b < NV; ++b) Rv(a, b) = fma(sa, z1[b], fma(pa, z2[b], Rv(a, b)));
      }
#pragma unroll 1
      for (int a = 0; a < NU; ++a) {
        const double sa = B.S[r][a], pa = B.P[r][a];
#pragma unroll
        for (int b = 0; b < NU; ++b) bb(a, b) = fma(sa, y1[b], fma(pa, y2[b], bb(a, b)));
      }
    }
  }

  }   // volume terms

  if (S.mode == OUT_ADJ_VOLUME) {
#pragma unroll 1
    for (int b = 0; b < NV; ++b)
#pragma unroll
      for (int a = 0; a < NV; ++a) S.vt[e + Eu * (a + NV * b)] = Rv(a, b);
#pragma unroll 1
    for (int b = 0; b < NU; ++b)
#pragma unroll
      for (int a = 0; a < NU; ++a) S.ut[e + Eu * (a + NU * b)] = bb(a, b);
    return;
  }

  // ---- source (src/rhs.jl:340-350), and the mass right-hand side to HBM
#pragma unroll 1
  for (int b = 0; b < NV && !adjoint; ++b)
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      const size_t l = (a + NV * b) * Eu + e;
      double x = Rv(a, b);
      if (F.mms_on) {
        x = fma(tf.cSP, F.PiSP[l], x);
        x = fma(tf.cB, F.PiBSP2[l], x);
        x = fma(tf.cC, F.PiCdiv[l], x);
        x = fma(tf.cD, F.PiDdiv[l], x);
      } else if (!F.src_on) {
        x += F.PiCdiv[l];
      }
      if (F.src_on) x = fma(tf.srct, F.srcP[l], x);
      F.mrhs[l] = x;
    }

  // ---- u-equation (src/rhs.jl:352-382): A_e UT = VB - Fu + e_1 V[0][0]
  if (!adjoint) {
    bb(0, 0) += S.xv[e];
  }
  // UT: in place of b (constant-coefficient kernels), in the space of R_v (general kernels: R_v is
  // spent once the mass right-hand side is written)
  Blk<NU, BT> UT = FAST ? bb : Blk<NU, BT>{smem + NU * NU * BT + tid};
  if constexpr (FAST) {
    // A_e = c² (K1 ⊗ I + I ⊗ K1) + e_0 e_0^T is diagonal in the eigenbasis Q ⊗ Q of K1 (whose
    // first eigenvector is e_0 with λ_0 = 0): UT = Q [ (Q^T b Q) ∘ L ] Q^T, L = 1/(c²(λ_i+λ_j)), 1 at (0,0).
    // Q[a][i] vanishes for a + i odd and in row and column 0 outside (0, 0): qnz skips those
    // terms at compile time. The four products run in place: a product with Q from the left
    // changes each column on its own, one from the right each row.
    const double ic2 = F.ic2e[e];
    if (eig) {
      if constexpr (NU != NV) {
      // as below, Ṽ accumulated column by column of V (padded with zeros to NU × NU): with
      // t = Q^T V[:, c], X += t ⊗ Q[c, :] (R_v's space is too small for Q^T V here)
#pragma unroll 1
      for (int i = 0; i < NU; ++i)
#pragma unroll
        for (int jj = 0; jj < NU; ++jj)
          if (i != 0 || jj != 0) bb(i, jj) = bb(i, jj) * (B.ilam2[i][jj] * ic2);
#pragma unroll 1
      for (int c = 0; c < NV; ++c) {
        double t[NU], x[NV];
#pragma unroll
        for (int a = 0; a < NV; ++a) x[a] = S.xv[e + Eu * (a + NV * c)];
#pragma unroll
        for (int i = 0; i < NU; ++i) t[i] = 0;
#pragma unroll
        for (int a = 0; a < NV; ++a)
#pragma unroll
          for (int i = 0; i < NU; ++i)
            if (qnz(a, i)) t[i] = fma(B.Q[a][i], x[a], t[i]);
#pragma unroll
        for (int i = 0; i < NU; ++i)
#pragma unroll
          for (int jj = 0; jj < NU; ++jj)
            if (qnz(c, jj) && (i != 0 || jj != 0)) bb(i, jj) = fma(t[i], B.Q[c][jj], bb(i, jj));
      }
      } else {
      // b is in the eigenbasis except for its volume part c²(K1 V + V K1), whose transform
      // c²(Λ Ṽ + Ṽ Λ), Ṽ = Q^T V Q, divided by c²(λ_i + λ_j) is Ṽ itself (zero at (0, 0)):
      // X = Ṽ + (Q^T b' Q) ∘ L. T1 = Q^T V by columns into the space of R_v (written out above),
      // then X = T1 Q + b' ∘ L by rows.
      Blk<NV, BT> T1 = Rv;
#pragma unroll 1
      for (int c = 0; c < NU; ++c) {
        double t[NU], x[NU];
#pragma unroll
        for (int a = 0; a < NU; ++a) x[a] = S.xv[e + Eu * (a + NU * c)];
#pragma unroll
        for (int i = 0; i < NU; ++i) t[i] = 0;
#pragma unroll
        for (int a = 0; a < NU; ++a)
#pragma unroll
          for (int i = 0; i < NU; ++i)
            if (qnz(a, i)) t[i] = fma(B.Q[a][i], x[a], t[i]);
#pragma unroll
        for (int i = 0; i < NU; ++i) T1(i, c) = t[i];
      }
#pragma unroll 1
      for (int i = 0; i < NU; ++i) {
        double t[NU];
#pragma unroll
        for (int jj = 0; jj < NU; ++jj) t[jj] = 0;
#pragma unroll
        for (int c = 0; c < NU; ++c) {
          const double x = T1(i, c);
#pragma unroll
          for (int jj = 0; jj < NU; ++jj)
            if (qnz(c, jj)) t[jj] = fma(x, B.Q[c][jj], t[jj]);
        }
#pragma unroll
        for (int jj = 0; jj < NU; ++jj)
          bb(i, jj) = (i == 0 && jj == 0) ? bb(0, 0) : fma(bb(i, jj), B.ilam2[i][jj] * ic2, t[jj]);
      }
      }
    } else {
#pragma unroll 1
    for (int c = 0; c < NU; ++c) {                 // T1 = Q^T b, by columns
      double t[NU];
#pragma unroll
      for (int i = 0; i < NU; ++i) t[i] = 0;
#pragma unroll
      for (int a = 0; a < NU; ++a) {
        const double x = bb(a, c);
#pragma unroll
        for (int i = 0; i < NU; ++i)
          if (qnz(a, i)) t[i] = fma(B.Q[a][i], x, t[i]);
      }
#pragma unroll
      for (int i = 0; i < NU; ++i) bb(i, c) = t[i];
    }
#pragma unroll 1
    for (int i = 0; i < NU; ++i) {                 // T2 = (T1 Q) ∘ L, by rows
      double t[NU];
#pragma unroll
      for (int jj = 0; jj < NU; ++jj) t[jj] = 0;
#pragma unroll
      for (int c = 0; c < NU; ++c) {
        const double x = bb(i, c);
#pragma unroll
        for (int jj = 0; jj < NU; ++jj)
          if (qnz(c, jj)) t[jj] = fma(x, B.Q[c][jj], t[jj]);
      }
#pragma unroll
      for (int jj = 0; jj < NU; ++jj) bb(i, jj) = (i == 0 && jj == 0) ? t[jj] : t[jj] * (B.ilam2[i][jj] * ic2);
    }
    }
#pragma unroll 1
    for (int jj = 0; jj < NU; ++jj) {              // T3 = Q T2, by columns
      double t[NU];
#pragma unroll
      for (int a = 0; a < NU; ++a) t[a] = 0;
#pragma unroll
      for (int i = 0; i < NU; ++i) {
        const double x = bb(i, jj);
#pragma unroll
        for (int a = 0; a < NU; ++a)
          if (qnz(a, i)) t[a] = fma(B.Q[a][i], x, t[a]);
      }
#pragma unroll
      for (int a = 0; a < NU; ++a) bb(a, jj) = t[a];
    }
#pragma unroll 1
    for (int a = 0; a < NU; ++a) {                 // UT = T3 Q^T, by rows
      double t[NU];
#pragma unroll
      for (int c = 0; c < NU; ++c) t[c] = 0;
#pragma unroll
      for (int jj = 0; jj < NU; ++jj) {
        const double x = bb(a, jj);
#pragma unroll
        for (int c = 0; c < NU; ++c)
          if (qnz(c, jj)) t[c] = fma(x, B.Q[c][jj], t[c]);
      }
#pragma unroll
      for (int c = 0; c < NU; ++c) bb(a, c) = t[c];
    }
  } else {
    // packed upper triangle of the symmetric inverse, by columns: entry (i, j), i ≤ j, in row j(j+1)/2 + i
    constexpr int n = NU * NU;
    double *X = &UT(0, 0), *bv = &bb(0, 0);       // UT and b as vectors a + NU c
#pragma unroll 1
    for (int i = 0; i < n; ++i) X[i * BT] = 0.0;
    // two columns jj, jj + 1 per pass: one read-modify-write of X[i] for both, twice the
    // independent loads of Ainv in flight
#pragma unroll 1
    for (int jj = 0; jj + 1 < n; jj += 2) {
      const double bj = bv[jj * BT], bk = bv[(jj + 1) * BT];
      const double *Aj = F.Ainv + (size_t)(jj * (jj + 1) / 2) * Eu + e;
      const double *Ak = Aj + (size_t)(jj + 1) * Eu;
      double sj = 0, sk = 0;
#pragma unroll 8
      for (int i = 0; i < jj; ++i) {
        const double a = Aj[(size_t)i * Eu], c = Ak[(size_t)i * Eu];
        const double bi = bv[i * BT];
        X[i * BT] = fma(c, bk, fma(a, bj, X[i * BT]));
        sj = fma(a, bi, sj);
        sk = fma(c, bi, sk);
      }
      // the 2 × 2 corner: (jj, jj), (jj, jj + 1), (jj + 1, jj + 1)
      const double ajj = Aj[(size_t)jj * Eu], ajk = Ak[(size_t)jj * Eu], akk = Ak[(size_t)(jj + 1) * Eu];
      X[jj * BT] = fma(ajk, bk, fma(ajj, bj, X[jj * BT] + sj));
      X[(jj + 1) * BT] = fma(akk, bk, fma(ajk, bj, X[(jj + 1) * BT] + sk));
    }
    if constexpr ((n & 1) != 0) {
      const int jj = n - 1;
      const double bj = bv[jj * BT];
      const double *Aj = F.Ainv + (size_t)(jj * (jj + 1) / 2) * Eu + e;
      double sj = 0;
#pragma unroll 4
      for (int i = 0; i < jj; ++i) {
        const double a = Aj[(size_t)i * Eu];
        X[i * BT] = fma(a, bj, X[i * BT]);
        sj = fma(a, bv[i * BT], sj);
      }
      X[jj * BT] = fma(Aj[(size_t)jj * Eu], bj, X[jj * BT] + sj);
    }
  }

  // ---- u outputs: RK4 (src/solver.jl:289-321): acc = k1 + 2 k2 + 2 k3 in this order, the next
  //      stage state u + c k, the last stage u + (dt/6)(acc + k4) with the finite check
  bool fin = true;
#pragma unroll 1
  for (int b = 0; b < NU; ++b)
#pragma unroll
    for (int a = 0; a < NU; ++a) {
      const size_t l = e + Eu * (a + NU * b);
      const double kk = UT(a, b);
      if (S.mode == OUT_RHS || S.mode == OUT_ADJ_USOLVE) {
        S.ut[l] = kk;
      } else if (S.mode == OUT_RK4_STAGE) {
        S.accu[l] = S.first ? kk : S.accu[l] + 2.0 * kk;
        S.su[l] = S.u0[l] + S.c * kk;
      } else if (S.mode == OUT_RK4_LAST) {
        // Chebyshev mode only: no error can arise after k_prep, so u is updated in place now
        const double x = S.u0[l] + S.c * (S.accu[l] + kk);
        S.uo[l] = x;
        fin = fin && isfinite(x);
      } else {
        S.accu[l] = S.accu[l] + kk;
      }
    }
  if (S.mode == OUT_RK4_LAST && !fin) atomicOr(F.nonfinite, 1u);
}

// Blocks per SM asked of k_stage: at low degrees the registers allow more than two blocks of
// 128 elements (the shared memory does), and the compiler keeps the kernel within them without
// spilling; from q_u = 4 on, two
__host__ __device__ constexpr int stage_m_blocks(int nu) { return nu <= 2 ? 5 : nu == 3 ? 4 : nu == 4 ? 3 : 2; }

template <int NU, int NV, bool FAST>
__global__ void __launch_bounds__(stage_threads(NU, NV, FAST), stage_m_blocks(NU))
    k_stage(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ Fields F,
            const __grid_constant__ StageIO S) {
  constexpr int BT = stage_threads(NU, NV, FAST);
  stage_body<NU, NV, FAST>(B, F, S, blockIdx.x * BT + (int)threadIdx.x, threadIdx.x);
}


// tile = stage_threads(NU, NV, FAST) elements per virtual block
template <int NU, int NV, bool FAST>
__global__ void __launch_bounds__(stage_threads(NU, NV, FAST), stage_m_blocks(NU))
    k_stage_m(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ MultiStage P) {
  for (int vb = blockIdx.x; vb < P.first[P.n]; vb += gridDim.x) {
    const int inst = multi_begin(P, vb);
    stage_body<NU, NV, FAST>(B, P.a[inst].F, P.a[inst].S, (vb - P.first[inst]) * P.tile + (int)threadIdx.x,
                             threadIdx.x);
  }
}

// ----------------------------------------------------------------------------
// The mass solve M(v_h) VT = R on every element (src/rhs.jl:778-951) and the v part of the outputs
// ----------------------------------------------------------------------------

// element of thread g: in the order of the Chebyshev step counts, or in mesh order
// (largest counts first: the blocks with the most work start first, and the short ones fill the
// SMs behind them). pref[b] = number of elements in the bins above b.
__device__ __forceinline__ int mass_element(const Fields &F, const StageIO &S, int g, int *pref) {
  if (!F.sorted) return g;
  int lo = NBIN - 1;
#pragma unroll 1
  for (int b = 0; b < NBIN; ++b)
    if (pref[b] <= g) { lo = b; break; }
  return F.bins[(size_t)lo * F.E + (g - pref[lo])];
}

// v outputs of modal entry l = e + E (a + NV b): RK4 as in k_stage (src/solver.jl:299-321)
__device__ __forceinline__ void store_v(const StageIO &S, size_t l, double kk, bool &fin) {
  if (S.mode == OUT_RHS) {
    S.vt[l] = kk;
  } else if (S.mode == OUT_RK4_STAGE) {
    S.accv[l] = S.first ? kk : S.accv[l] + 2.0 * kk;
    S.sv[l] = S.v0[l] + S.c * kk;
  } else if (S.mode == OUT_RK4_LAST) {
    const double x = S.v0[l] + S.c * (S.accv[l] + kk);
    S.vo[l] = x;
    fin = fin && isfinite(x);
  } else {
    S.accv[l] = S.accv[l] + kk;
  }
}

// The mass solves run on a team of threads per element. One step of either solver costs one
// application of K = P_h^T diag(G W) P_h (G = 2βv at the high-order points, W = w_h w_h^T their
// weights, folded into PhW) to a vector of NV² modal entries, and its FP64 work is cut across
// the team by rows of the point grid: unit u of the team takes the mirrored rows u and QH-1-u
// (the middle row alone when QH is odd), takes them to the points and back (phase 1), and leaves
// for each mode column b the sum and the difference of the two rows' results in shared memory;
// then every thread finishes J of the NV² modal entries from the units' rows (phase 2), for
// which it also keeps the solver's vectors. A team lives in one warp, so its phases are ordered
// by __syncwarp on the team's lanes. Spreading an element over the team matters because one
// warp is tied to one SM sub-partition, whose FP64 rate is a small fraction of a lane per clock:
// with one element per thread, the warps of the elements with the most steps ran for many times
// the average and left the SMs idle behind them.
template <int NU, int NV>
struct ChebTeam {
  static constexpr int QH = qhigh(NU, NV);
  static constexpr int U = QH / 2 + (QH & 1);          // team size: row pairs (+ the middle row)
  static constexpr int TPW = 32 / U;                    // teams per warp
  static constexpr int TPB = TPW * (CHEB_THREADS / 32); // elements per block
  static constexpr int NE = NV * NV;
  static constexpr int J = (NE + U - 1) / U;            // modal entries per thread
  static constexpr int SLOT = NE + 2 * U * NV;          // x, then the row sums and differences
};

// The shared setup of a team kernel: Ph and PhW in shared memory, the team of this thread, its
// unit, its lanes. Returns false for lanes without a team.
struct TeamPos {
  int slot, u;
  unsigned mask;
};
template <int NU, int NV>
__device__ __forceinline__ bool team_pos(TeamPos &P) {
  using T = ChebTeam<NU, NV>;
  const int lane = threadIdx.x & 31, tw = lane / T::U;
  if (tw >= T::TPW) return false;
  P.u = lane - tw * T::U;
  P.slot = (threadIdx.x >> 5) * T::TPW + tw;
  P.mask = ((1u << T::U) - 1u) << (tw * T::U);
  return true;
}

// Σ over the team's lanes of x, in the order of the units, on every lane of the team
template <int U>
__device__ __forceinline__ double team_sum(double x, unsigned mask) {
  const int base = __ffs(mask) - 1;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < U; ++i) s += __shfl_sync(mask, x, base + i);
  return s;
}

// acc[j] ± (K x)[k_j] on the thread's entries k_j = u + U j (+ with SIGN = 1, - with -1), for x in
// the team's shared slot xs (complete, after a __syncwarp). zs, zd hold the units' row results
// until the next __syncwarp of the caller.
template <int NU, int NV, int SIGN>
__device__ __forceinline__ void team_K(const Basis<NU, NV> &B, const Fields &F, size_t Eu, int e, int u,
                                       unsigned mask, const double *Phs, const double *PhWs, const double *xs,
                                       double *zs, double *zd, double (&acc)[ChebTeam<NU, NV>::J]) {
  using T = ChebTeam<NU, NV>;
  constexpr int QH = T::QH, U = T::U, NE = T::NE, J = T::J;
  const int r1 = u, r2 = QH - 1 - u;                    // the unit's rows (r1 = r2 for the middle row)
  auto rowZ = [&](const double (&Tv)[NV], int r, double (&Z)[NV]) {
    double Y[QH];
    ph_to_points<QH, NV>(B.Ph, Tv, Y);
#pragma unroll
    for (int s2 = 0; s2 < QH; ++s2) Y[s2] *= F.G[(r + QH * s2) * Eu + e];
    ph_from_points<QH, NV>(B.PhW, Y, Z);
  };
  // phase 1: rows r1, r2 of P_h x, at the points, weighted, back to the modes
  {
    double Tp[NV], Tm[NV], Zp[NV], Zm[NV];
#pragma unroll
    for (int b = 0; b < NV; ++b) {
      double ev = 0.0, od = 0.0;
#pragma unroll
      for (int a = 0; a < NV; a += 2) ev = fma(Phs[r1 * NV + a], xs[a + NV * b], ev);
#pragma unroll
      for (int a = 1; a < NV; a += 2) od = fma(Phs[r1 * NV + a], xs[a + NV * b], od);
      Tp[b] = ev + od;
      Tm[b] = ev - od;
    }
    rowZ(Tp, r1, Zp);
    rowZ(Tm, r2, Zm);
#pragma unroll
    for (int b = 0; b < NV; ++b) {
      zs[u * NV + b] = r1 == r2 ? Zp[b] : Zp[b] + Zm[b];
      zd[u * NV + b] = Zp[b] - Zm[b];
    }
  }
  __syncwarp(mask);
  // phase 2: the thread's entries
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = u + U * j;
    if (k < NE) {
      const int a = k % NV, b = k / NV;
      const double *z = ((a & 1) ? zd : zs) + b;
      double x = acc[j];
#pragma unroll
      for (int v = 0; v < U; ++v) x = fma(SIGN * PhWs[v * NV + a], z[v * NV], x);
      acc[j] = x;
    }
  }
}

// Shared memory of a team kernel and its setup: the bin prefix (sorted order) and the bases;
// g0 is the first element slot of the block (slots in the order of mass_element)
#define WEDG_TEAM_SETUP(g0)                                                                     \
  using T = ChebTeam<NU, NV>;                                                                   \
  constexpr int U = T::U, NE = T::NE, J = T::J;                                                 \
  __shared__ double sh[T::TPB * T::SLOT];                                                       \
  __shared__ double Phs[T::QH * NV], PhWs[T::QH * NV];                                          \
  __shared__ int pref[NBIN];                                                                    \
  for (int i = threadIdx.x; i < T::QH * NV; i += blockDim.x) {                                 \
    Phs[i] = B.Ph[i / NV][i % NV];                                                              \
    PhWs[i] = B.PhW[i / NV][i % NV];                                                            \
  }                                                                                             \
  if (F.sorted && threadIdx.x == 0) {                                                           \
    int acc_ = 0;                                                                               \
    for (int b = NBIN - 1; b >= 0; --b) { pref[b] = acc_; acc_ += F.bin_count[S.parity * NBIN + b]; } \
  }                                                                                             \
  __syncthreads();                                                                              \
  TeamPos tp;                                                                                   \
  if (!team_pos<NU, NV>(tp)) return;                                                            \
  const int g = (g0) + tp.slot;                                                                 \
  if (g >= F.E) return;                                                                         \
  if (err_word(F) != ERR_NONE) return;                                                          \
  const int u = tp.u;                                                                           \
  const unsigned tmask = tp.mask;                                                               \
  const size_t Eu = (size_t)F.E;                                                                \
  double *xs = sh + tp.slot * T::SLOT, *zs = xs + NE, *zd = zs + U * NV;                        \
  (void)Eu;

// k_cheb: the Chebyshev mass solve (Saad Alg. 12.1, src/rhs.jl:920-939). Elements are visited in
// decreasing order of their step counts (k_prep lists them by count), so the longest solves start
// first. The team keeps the residual r, the iterate X and the direction d of its entries in
// registers and d in its shared slot.
template <int NU, int NV>
__device__ __forceinline__ void cheb_body(const Basis<NU, NV> &B, const Fields &F, const StageIO &S, int g0) {
  WEDG_TEAM_SETUP(g0);
  const int e = mass_element(F, S, g, pref);
  const double th = F.th[e], de = F.de[e];
  const double s1 = th / de;
  const int n = F.cheb_common ? F.nmax[S.parity] : F.nst[e];
  const double ith = 1.0 / th;
  double rr[J], xx[J], dd[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = u + U * j;
    rr[j] = xx[j] = dd[j] = 0.0;
    if (k < NE) {
      const double x = F.mrhs[k * Eu + e];
      rr[j] = x;
      dd[j] = x * ith;
      xs[k] = dd[j];
    }
  }
  __syncwarp(tmask);
  double rho = 1.0 / s1;
#pragma unroll 1
  for (int step = 1; step <= n; ++step) {
#pragma unroll
    for (int j = 0; j < J; ++j) {
      xx[j] += dd[j];
      rr[j] -= dd[j];
    }
    if (step == n) break;
    team_K<NU, NV, 1>(B, F, Eu, e, u, tmask, Phs, PhWs, xs, zs, zd, rr);   // r += K d
    const double rhon = 1.0 / (2.0 * s1 - rho);
    const double c1 = rhon * rho, c2 = 2.0 * rhon / de;
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int k = u + U * j;
      if (k < NE) {
        dd[j] = fma(c1, dd[j], c2 * rr[j]);
        xs[k] = dd[j];
      }
    }
    rho = rhon;
    __syncwarp(tmask);
  }

  bool fin = true;
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = u + U * j;
    if (k < NE) store_v(S, e + Eu * k, xx[j], fin);
  }
  if (S.mode == OUT_RK4_LAST && !fin) atomicOr(F.nonfinite, 1u);
}

// k_cg: the mass solve by conjugate gradients from X = R (src/rhs.jl:821-853), elements in mesh
// order. The team first forms G = 2βv at the high-order points of its rows (each unit reads only
// the rows it wrote), then iterates with p in its shared slot and the inner products summed over
// the team's lanes in a fixed order, so that every lane takes the same decisions.
template <int NU, int NV>
__device__ __forceinline__ void cg_body(const Basis<NU, NV> &B, const Fields &F, const StageIO &S, int g0) {
  WEDG_TEAM_SETUP(g0);
  constexpr int QH = T::QH;
  const int e = g;
  {
    // G rows u and QH-1-u of this element
    const int r1 = u, r2 = QH - 1 - u;
    auto vx = [&](int a, int b) { return S.xv[e + Eu * (a + NV * b)]; };
    double Tp[NV], Tm[NV];
    ph_row_pair<QH, NV>(B.Ph, r1, vx, Tp, Tm);
    auto gput = [&](const double (&Tv)[NV], int r) {
      double Y[QH];
      ph_to_points<QH, NV>(B.Ph, Tv, Y);
#pragma unroll
      for (int s2 = 0; s2 < QH; ++s2) {
        const size_t gi = (r + QH * s2) * Eu + e;
        F.G[gi] = Y[s2] * F.beta2[gi];
      }
    };
    gput(Tp, r1);
    if (r2 != r1) gput(Tm, r2);
  }
  double X[J], r[J], p[J], Ap[J];
  double r0 = 0;
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = u + U * j;
    X[j] = r[j] = p[j] = 0.0;
    if (k < NE) {
      const double x = F.mrhs[k * Eu + e];
      X[j] = x;
      xs[k] = x;
      r0 = fma(x, x, r0);
    }
  }
  r0 = sqrt(team_sum<U>(r0, tmask));
  __syncwarp(tmask);
  team_K<NU, NV, 1>(B, F, Eu, e, u, tmask, Phs, PhWs, xs, zs, zd, r);    // r = R - M X = K R for X = R
  double rr = 0;
#pragma unroll
  for (int j = 0; j < J; ++j) {
    p[j] = r[j];
    rr = fma(r[j], r[j], rr);
  }
  rr = team_sum<U>(rr, tmask);
  const int maxit = NV * NV + 10;
  int it = 0;
  bool bad = false;
  while (sqrt(rr) > F.mass_tol * r0 && it < maxit) {
    ++it;
    __syncwarp(tmask);                              // the last phase 2 has read zs, zd
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int k = u + U * j;
      if (k < NE) xs[k] = p[j];
    }
    __syncwarp(tmask);
#pragma unroll
    for (int j = 0; j < J; ++j) Ap[j] = p[j];
    team_K<NU, NV, -1>(B, F, Eu, e, u, tmask, Phs, PhWs, xs, zs, zd, Ap);  // A p = p - K p
    double pAp = 0;
#pragma unroll
    for (int j = 0; j < J; ++j) pAp = fma(p[j], Ap[j], pAp);
    pAp = team_sum<U>(pAp, tmask);
    if (!(pAp > 0.0)) { bad = true; break; }
    const double al = rr / pAp;
    double rrn = 0;
#pragma unroll
    for (int j = 0; j < J; ++j) {
      X[j] = fma(al, p[j], X[j]);
      r[j] = fma(-al, Ap[j], r[j]);
      rrn = fma(r[j], r[j], rrn);
    }
    rrn = team_sum<U>(rrn, tmask);
    const double bt = rrn / rr;
#pragma unroll
    for (int j = 0; j < J; ++j) p[j] = fma(bt, p[j], r[j]);
    rr = rrn;
  }
  if (bad) {
    if (u == 0) atomicMin(F.err, (1ull << ERR_CLASS_SHIFT) | (unsigned long long)(e + 1));
    return;
  }
  if (u == 0 && sqrt(rr) > F.mass_tol * r0) atomicAdd(F.cg_nfail, 1u);

  bool fin = true;
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = u + U * j;
    if (k < NE) store_v(S, e + Eu * k, X[j], fin);
  }
  if (S.mode == OUT_RK4_LAST && !fin) atomicOr(F.nonfinite, 1u);
}

#undef WEDG_TEAM_SETUP

// The team kernels: a block of `threads` takes (threads / 32) teams per warp of elements
template <int NU, int NV>
__device__ __forceinline__ int team_tile() {
  return (int)(blockDim.x >> 5) * ChebTeam<NU, NV>::TPW;
}

template <int NU, int NV>
__global__ void __launch_bounds__(CHEB_THREADS, 3)
    k_cheb(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ Fields F,
           const __grid_constant__ StageIO S) {
  cheb_body<NU, NV>(B, F, S, blockIdx.x * team_tile<NU, NV>());
}

template <int NU, int NV>
__global__ void __launch_bounds__(CHEB_THREADS, 3)
    k_cg(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ Fields F,
         const __grid_constant__ StageIO S) {
  cg_body<NU, NV>(B, F, S, blockIdx.x * team_tile<NU, NV>());
}

// tile = team_tile elements per virtual block; CG selects k_cg's body
template <int NU, int NV, bool CG>
__global__ void __launch_bounds__(CHEB_THREADS, 3)
    k_mass_m(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ MultiStage P) {
  for (int vb = blockIdx.x; vb < P.first[P.n]; vb += gridDim.x) {
    const int inst = multi_begin(P, vb);
    const int g0 = (vb - P.first[inst]) * P.tile;
    if constexpr (CG) cg_body<NU, NV>(B, P.a[inst].F, P.a[inst].S, g0);
    else cheb_body<NU, NV>(B, P.a[inst].F, P.a[inst].S, g0);
  }
}

// Last RK4 update when the last stage may still raise an error inside k_cg
// (CG mode): u += (dt/6) acc unless an error was recorded.
__global__ void k_rk4_final(int n_u, int n_v, double *u, double *v, const double *accu, const double *accv,
                            double c, const unsigned long long *err, unsigned int *nonfinite);

// Device-side step bookkeeping after each RK4 step: counts completed steps and,
// when asked, stops the run after a non-finite result.
__global__ void k_step_done(unsigned long long *err, const unsigned int *nonfinite, int stop_nonfinite,
                            long long *steps_done);

}  // namespace wedg

#include "wedg_adjoint.cuh"

