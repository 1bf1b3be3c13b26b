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
//   k_mass   the mass solve (Chebyshev :920-939 or CG :821-853) and the v part
//            of the RK4 update. Elements are visited in the order of their
//            Chebyshev step counts (k_prep lists them by count), so the lanes
//            of a warp run the same number of steps.
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
//   beta, G     [(r + QH s) E + e]
//   mass rhs    [(a + NV b) E + e]
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace wedg {

constexpr unsigned long long ERR_NONE = ~0ull;
constexpr int ERR_CLASS_SHIFT = 56;   // class 0: boundary weight, 1: mass matrix not PD, 3: stopped (non-finite)
constexpr int NBIN = 48;              // Chebyshev-count bins of the mass kernel (the last holds n ≥ NBIN)
constexpr int MASS_THREADS = 64;

__host__ __device__ constexpr int qhigh(int nu, int nv) {
  // q_high = max(ceil(3 q_v / 2) + 1, q_u + 1), src/solver.jl:483
  return ((3 * (nv - 1) + 1) / 2 + 1) > nu ? ((3 * (nv - 1) + 1) / 2 + 1) : nu;
}

// threads per block of k_stage: the element arrays (2 NU² + 2 NV² doubles per
// thread) must fit the 227 KB of shared memory of one block
__host__ __device__ constexpr int stage_threads(int nu, int nv) {
  return 128 * (2 * nu * nu + 2 * nv * nv) * 8 <= 232448 ? 128 : 96;
}

template <int NU, int NV>
struct Basis {
  static constexpr int NQ = NU;
  static constexpr int QH = qhigh(NU, NV);
  double w[NQ];
  double P[NQ][NU], S[NQ][NU];   // P[i][d] = P_u[i, d], S likewise; the v-basis is d < NV
  double El[NU], Er[NU], E1l[NU], E1r[NU];
  double Ph[QH][NV];             // P_h_v[r, d]
  double Wh[QH][QH];             // W2d_h[r, s]
  double K1[NU][NU];             // 1D stiffness S^T diag(w) S
  double Q[NU][NU];              // its eigenvectors, Q[row][col]; Q[.][0] = e_0
  double ilam2[NU][NU];          // 1 / (λ_i + λ_j), and 1 at (0, 0)
};

struct Fields {
  int N, E;
  const double *Cw, *Aw, *Ainv, *ic2e, *c2e, *ae;
  const double *hc2, *haf, *hcf, *hbf, *hc2m, *hafm, *hJC;
  const double *vc2, *vaf, *vcf, *vbf, *vc2m, *vafm, *vJC;
  const double *bsp[4], *bspn[4];
  const double *PiSP, *PiBSP2, *PiCdiv, *PiDdiv, *srcP;
  const double *beta;
  double *tr, *G, *th, *de;
  double *mrhs;               // right-hand side of the mass system, [(a + NV b) E + e]
  int *nst, *nmax;
  int *bins, *bin_count;      // elements by Chebyshev count: bins[b E + i], two count buffers of NBIN
  unsigned long long *nsum;   // Σ of the per-element Chebyshev step counts
  unsigned long long *err;
  unsigned int *cg_nfail, *nonfinite;
  double theta, tau, lu, lv, omega, two_h, four_hh, mass_tol, Lcheb;
  int one_sided, mms_on, src_on, cg, cheb_common, sorted;
  int kind[4];
  double gam[4], eta[4], sig[4], kb[4], kap[4];
};

enum StageMode { OUT_RHS = 0, OUT_RK4_STAGE = 1, OUT_RK4_LAST = 2, OUT_RK4_LAST_ACC = 3 };

struct StageIO {
  const double *xu, *xv;     // stage state
  double ct, st, srct;       // time factors of the stage (src/rhs.jl:509-511)
  double cSP, cB, cC, cD;    // source weights: -ω²ct, -2ω³ st ct, 1 - ct, ω st
  int mode, first;
  int parity;                // which bin-count buffer this stage fills (the other is cleared)
  double *ut, *vt;           // OUT_RHS
  const double *u0, *v0;     // RK4 base state
  double *su, *sv;           // next stage state
  double *accu, *accv;       // k1 + 2k2 + 2k3 (+ k4)
  double *uo, *vo;           // in-place target of the last stage
  double c;                  // next-stage factor, or dt/6 on the last stage
};

__device__ __forceinline__ unsigned long long err_word(const Fields &F) {
  return *(volatile unsigned long long *)F.err;
}

// A thread-private n×n block in shared memory: X(a, b) at base[(a + n b) BT + tid]
template <int n, int BT>
struct Blk {
  double *p;
  __device__ __forceinline__ double &operator()(int a, int b) const { return p[(a + n * b) * BT]; }
};

// ----------------------------------------------------------------------------
// k_prep: traces, boundary weight check, Chebyshev interval data
// ----------------------------------------------------------------------------

// Traces of an n×n block X on the four sides (src/rhs.jl:388-410):
//   oB[i] = Σ_b P[i,b] Σ_a El[a] X[a][b],  oT with Er,
//   oL[i] = Σ_b P[i,b] Σ_a El[a] X[b][a],  oR with Er.
template <int NQ, int NU, int n>
__device__ __forceinline__ void trace4(const double (&X)[n][n], const double (&P)[NQ][NU], const double *El,
                                       const double *Er, double *tr, int fam, int E, int e) {
  double sB[n], sT[n], sL[n], sR[n];
#pragma unroll
  for (int b = 0; b < n; ++b) {
    double xb = 0, xt = 0, yl = 0, yr = 0;
#pragma unroll
    for (int a = 0; a < n; ++a) {
      xb = fma(El[a], X[a][b], xb);
      xt = fma(Er[a], X[a][b], xt);
      yl = fma(El[a], X[b][a], yl);
      yr = fma(Er[a], X[b][a], yr);
    }
    sB[b] = xb; sT[b] = xt; sL[b] = yl; sR[b] = yr;
  }
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    double oB = 0, oT = 0, oL = 0, oR = 0;
#pragma unroll
    for (int b = 0; b < n; ++b) {
      oB = fma(P[i][b], sB[b], oB);
      oT = fma(P[i][b], sT[b], oT);
      oL = fma(P[i][b], sL[b], oL);
      oR = fma(P[i][b], sR[b], oR);
    }
    tr[((fam * 4 + 0) * NQ + i) * (size_t)E + e] = oB;
    tr[((fam * 4 + 1) * NQ + i) * (size_t)E + e] = oT;
    tr[((fam * 4 + 2) * NQ + i) * (size_t)E + e] = oL;
    tr[((fam * 4 + 3) * NQ + i) * (size_t)E + e] = oR;
  }
}

template <int n>
__device__ __forceinline__ void load_regs(double (&X)[n][n], const double *x, int E, int e) {
#pragma unroll
  for (int b = 0; b < n; ++b)
#pragma unroll
    for (int a = 0; a < n; ++a) X[a][b] = x[e + (size_t)E * (a + n * b)];
}

template <int NU, int NV>
__global__ void __launch_bounds__(128) k_prep(const __grid_constant__ Basis<NU, NV> B,
                                              const __grid_constant__ Fields F,
                                              const __grid_constant__ StageIO S) {
  constexpr int NQ = NU, QH = Basis<NU, NV>::QH;
  const int E = F.E, N = F.N;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int j = e % N, k = e / N;
  if (e < NBIN && F.sorted) F.bin_count[(1 - S.parity) * NBIN + e] = 0;   // for the next stage
  {
    double U[NU][NU];
    load_regs<NU>(U, S.xu, E, e);
    trace4<NQ, NU, NU>(U, B.P, B.E1l, B.E1r, F.tr, 0, E, e);
  }
  double V[NV][NV];
  load_regs<NV>(V, S.xv, E, e);
  trace4<NQ, NU, NV>(V, B.P, B.El, B.Er, F.tr, 1, E, e);
  trace4<NQ, NU, NV>(V, B.P, B.E1l, B.E1r, F.tr, 2, E, e);

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
      const double v_fp = F.tr[((1 * 4 + s) * NQ + i) * (size_t)E + e];
      const double v_ex = -F.omega * S.st * F.bsp[s][m + (size_t)N * i];
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
  // Chebyshev interval of the element: v_q = P_h V P_h^T, G = 2βv_q, a± = 1 - extrema(G)
  double gmin = 1.0 / 0.0, gmax = -1.0 / 0.0;
  bool nan = false;
#pragma unroll 1
  for (int r = 0; r < QH; ++r) {
    double T[NV];
#pragma unroll
    for (int b = 0; b < NV; ++b) {
      double t = 0;
#pragma unroll
      for (int a = 0; a < NV; ++a) t = fma(B.Ph[r][a], V[a][b], t);
      T[b] = t;
    }
#pragma unroll 2
    for (int s2 = 0; s2 < QH; ++s2) {
      double g = 0;
#pragma unroll
      for (int b = 0; b < NV; ++b) g = fma(T[b], B.Ph[s2][b], g);
      const size_t gi = (r + QH * s2) * (size_t)E + e;
      g = g * (2.0 * F.beta[gi]);
      nan |= (g != g);
      gmin = fmin(gmin, g);
      gmax = fmax(gmax, g);
      F.G[gi] = g * B.Wh[r][s2];
    }
  }
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
    atomicMax(F.nmax, nw);
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

// ----------------------------------------------------------------------------
// k_stage helpers
// ----------------------------------------------------------------------------

// Numerical flux slots A, D, F at point i of side s of the element
// (src/rhs.jl:620-700 for interior faces, :65-103 and :738-763 for physical sides).
template <int NU, int NV>
__device__ __forceinline__ void side_point(const Basis<NU, NV> &B, const Fields &F, const StageIO &S, int s,
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
    const double v_fp = T(1, s, e);
    const double gun = sgn * (F.two_h * T(0, s, e));
    const double gvn = sgn * (F.two_h * T(2, s, e));
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
  const double th = F.theta, tau = F.tau, two_h = F.two_h;
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
  if (F.one_sided) {
    const double c2m = c2m_a[fi], c2p = c2p_a[fi], afm = afm_a[fi], afp = afp_a[fi], K = jc_a[fi];
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
    const double c2 = c2p_a[fi], af = afp_a[fi];
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

// ----------------------------------------------------------------------------
// k_stage: fluxes, lifts, volume, source, u-equation; the mass right-hand side to HBM
// ----------------------------------------------------------------------------
template <int NU, int NV, bool FAST>
__global__ void __launch_bounds__(stage_threads(NU, NV), 1)
    k_stage(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ Fields F,
            const __grid_constant__ StageIO S) {
  constexpr int NQ = NU, BT = stage_threads(NU, NV);
  extern __shared__ double smem[];
  const int tid = threadIdx.x;
  const int E = F.E, N = F.N;
  const int e = blockIdx.x * BT + tid;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int j = e % N, k = e / N;
  const double two_h = F.two_h, four_hh = F.four_hh;
  // thread-private blocks: X1, X2 (NU²), Y1, Y2 (NV²)
  Blk<NU, BT> X1{smem + tid}, X2{smem + NU * NU * BT + tid};
  Blk<NV, BT> Y1{smem + 2 * NU * NU * BT + tid}, Y2{smem + (2 * NU * NU + NV * NV) * BT + tid};
  Blk<NU, BT> Ub = X1, bb = X2;     // U (volume), u-equation right-hand side b
  Blk<NV, BT> Vb = Y1, Rv = Y2;     // V, v-equation right-hand side

  // ---- faces and lifts (src/rhs.jl:421-473): Rv (v-equation), b = -Fu (u-equation)
#pragma unroll 1
  for (int a = 0; a < NV; ++a)
#pragma unroll
    for (int b = 0; b < NV; ++b) Rv(a, b) = 0.0;
#pragma unroll 1
  for (int a = 0; a < NU; ++a)
#pragma unroll
    for (int b = 0; b < NU; ++b) bb(a, b) = 0.0;
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    const bool boundary = (s == 0 && j == 0) || (s == 1 && j == N - 1) || (s == 2 && k == 0) || (s == 3 && k == N - 1);
    double YA[NV], YD[NV], YF[NU];
#pragma unroll
    for (int b = 0; b < NU; ++b) {
      if (b < NV) { YA[b] = 0.0; YD[b] = 0.0; }
      YF[b] = 0.0;
    }
#pragma unroll 1
    for (int i = 0; i < NQ; ++i) {
      double A, D, Fs;
      side_point<NU, NV>(B, F, S, s, boundary, j, k, e, i, A, D, Fs);
      const double wa = B.w[i] * A, wd = B.w[i] * D, wf = B.w[i] * Fs;
#pragma unroll
      for (int b = 0; b < NU; ++b) {
        if (b < NV) {
          YA[b] = fma(B.P[i][b], wa, YA[b]);
          YD[b] = fma(B.P[i][b], wd, YD[b]);
        }
        YF[b] = fma(B.P[i][b], wf, YF[b]);
      }
    }
    const double *Ev = (s == 0 || s == 2) ? B.El : B.Er;
    const double *E1 = (s == 0 || s == 2) ? B.E1l : B.E1r;
    if (s < 2) {
#pragma unroll 1
      for (int a = 0; a < NV; ++a) {
        const double ca = two_h * Ev[a], cd = four_hh * E1[a];
#pragma unroll
        for (int b = 0; b < NV; ++b) Rv(a, b) = fma(cd, YD[b], fma(ca, YA[b], Rv(a, b)));
      }
#pragma unroll 1
      for (int a = 0; a < NU; ++a) {
        const double ce = -E1[a];
#pragma unroll
        for (int b = 0; b < NU; ++b) bb(a, b) = fma(ce, YF[b], bb(a, b));
      }
    } else {
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const double ca = two_h * YA[a], cd = four_hh * YD[a];
#pragma unroll
        for (int b = 0; b < NV; ++b) Rv(a, b) = fma(cd, E1[b], fma(ca, Ev[b], Rv(a, b)));
      }
#pragma unroll
      for (int a = 0; a < NU; ++a) {
        const double ce = -YF[a];
#pragma unroll
        for (int b = 0; b < NU; ++b) bb(a, b) = fma(ce, E1[b], bb(a, b));
      }
    }
  }

  // ---- state of the stage
  const size_t Eu = (size_t)E;
#pragma unroll 1
  for (int b = 0; b < NV; ++b)
#pragma unroll
    for (int a = 0; a < NV; ++a) Vb(a, b) = S.xv[e + Eu * (a + NV * b)];
#pragma unroll 1
  for (int b = 0; b < NU; ++b)
#pragma unroll
    for (int a = 0; a < NU; ++a) Ub(a, b) = S.xu[e + Eu * (a + NU * b)];

  // ---- volume terms (src/rhs.jl:309-333): Rv += -4/h² [(c²∇φ_v,∇u_h) + (α∇φ_v,∇v_h)],
  //      b += (c²∇φ_u, ∇v_h)
  if constexpr (FAST) {
    // constant c², α on the element: Cw = c² W, Aw = α W, so that with the
    // 1D stiffness K1 = S^T diag(w) S and the orthonormality of the basis
    //   (c²∇φ_v, ∇u_h) = c² (K1 U + U K1)[v-block],  (α∇φ_v, ∇v_h) = α (K1 V + V K1)
    //   (c²∇φ_u, ∇v_h) = c² (K1[:, v] V + V K1[v, :])
    // (row and column 0 of K1 vanish: the derivative of the constant mode is 0).
    // Each output row is built at once, so the FMAs of a row are independent.
    const double c2 = F.c2e[e], al = F.ae[e];
    const double mc2 = -four_hh * c2, mal = -four_hh * al;
#pragma unroll 1
    for (int a = 0; a < NV; ++a) {
      double su[NV], sv[NV];
#pragma unroll
      for (int b = 0; b < NV; ++b) { su[b] = 0.0; sv[b] = 0.0; }
#pragma unroll
      for (int c = 1; c < NU; ++c) {
        const double kac = B.K1[a][c], uac = Ub(a, c);
#pragma unroll
        for (int b = 0; b < NV; ++b) su[b] = fma(kac, Ub(c, b), fma(uac, B.K1[c][b], su[b]));
      }
#pragma unroll
      for (int c = 1; c < NV; ++c) {
        const double kac = B.K1[a][c], vac = Vb(a, c);
#pragma unroll
        for (int b = 0; b < NV; ++b) sv[b] = fma(kac, Vb(c, b), fma(vac, B.K1[c][b], sv[b]));
      }
#pragma unroll
      for (int b = 0; b < NV; ++b) Rv(a, b) = fma(mc2, su[b], fma(mal, sv[b], Rv(a, b)));
    }
#pragma unroll 1
    for (int a = 0; a < NU; ++a) {
      double s1[NU];
#pragma unroll
      for (int b = 0; b < NU; ++b) s1[b] = 0.0;
#pragma unroll
      for (int c = 1; c < NV; ++c) {
        const double kac = B.K1[a][c];
#pragma unroll
        for (int b = 0; b < NV; ++b) s1[b] = fma(kac, Vb(c, b), s1[b]);
      }
      if (a < NV) {
#pragma unroll
        for (int c = 1; c < NV; ++c) {
          const double vac = Vb(a, c);
#pragma unroll
          for (int b = 0; b < NU; ++b) s1[b] = fma(vac, B.K1[c][b], s1[b]);
        }
      }
#pragma unroll
      for (int b = 0; b < NU; ++b) bb(a, b) = fma(c2, s1[b], bb(a, b));
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
        for (int b = 0; b < NU; ++b) { const double x = Ub(a, b); tu1[b] = fma(sa, x, tu1[b]); tu2[b] = fma(pa, x, tu2[b]); }
        if (a < NV) {
#pragma unroll
          for (int b = 0; b < NV; ++b) { const double x = Vb(a, b); tv1[b] = fma(sa, x, tv1[b]); tv2[b] = fma(pa, x, tv2[b]); }
        }
      }
      // the row at the points: g1[s] = Σ_b tu1[b] P[s][b], ... (independent over s)
      double g1[NQ], g2[NQ], gv1[NQ], gv2[NQ];
#pragma unroll
      for (int s2 = 0; s2 < NQ; ++s2) { g1[s2] = 0; g2[s2] = 0; gv1[s2] = 0; gv2[s2] = 0; }
#pragma unroll
      for (int b = 0; b < NU; ++b) {
#pragma unroll
        for (int s2 = 0; s2 < NQ; ++s2) {
          g1[s2] = fma(tu1[b], B.P[s2][b], g1[s2]);
          g2[s2] = fma(tu2[b], B.S[s2][b], g2[s2]);
          if (b < NV) {
            gv1[s2] = fma(tv1[b], B.P[s2][b], gv1[s2]);
            gv2[s2] = fma(tv2[b], B.S[s2][b], gv2[s2]);
          }
        }
      }
      double z1[NV], z2[NV], y1[NU], y2[NU];
#pragma unroll
      for (int b = 0; b < NV; ++b) { z1[b] = 0; z2[b] = 0; }
#pragma unroll
      for (int b = 0; b < NU; ++b) { y1[b] = 0; y2[b] = 0; }
#pragma unroll
      for (int s2 = 0; s2 < NQ; ++s2) {
        const size_t ci = (r + NQ * s2) * Eu + e;
        const double cw = F.Cw[ci], aw = F.Aw[ci];
        const double h1 = fma(aw, gv1[s2], cw * g1[s2]), h2 = fma(aw, gv2[s2], cw * g2[s2]);
        const double b1 = cw * gv1[s2], b2 = cw * gv2[s2];
#pragma unroll
        for (int b = 0; b < NV; ++b) { z1[b] = fma(h1, B.P[s2][b], z1[b]); z2[b] = fma(h2, B.S[s2][b], z2[b]); }
#pragma unroll
        for (int b = 0; b < NU; ++b) { y1[b] = fma(b1, B.P[s2][b], y1[b]); y2[b] = fma(b2, B.S[s2][b], y2[b]); }
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

  // ---- source (src/rhs.jl:340-350), and the mass right-hand side to HBM
#pragma unroll 1
  for (int b = 0; b < NV; ++b)
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      const size_t l = (a + NV * b) * Eu + e;
      double x = Rv(a, b);
      if (F.mms_on) {
        x = fma(S.cSP, F.PiSP[l], x);
        x = fma(S.cB, F.PiBSP2[l], x);
        x = fma(S.cC, F.PiCdiv[l], x);
        x = fma(S.cD, F.PiDdiv[l], x);
      } else if (!F.src_on) {
        x += F.PiCdiv[l];
      }
      if (F.src_on) x = fma(S.srct, F.srcP[l], x);
      F.mrhs[l] = x;
    }

  // ---- u-equation (src/rhs.jl:352-382): A_e UT = VB - Fu + e_1 V[0][0]; UT into X1 (U is dead)
  bb(0, 0) += Vb(0, 0);
  Blk<NU, BT> UT = X1;
  if constexpr (FAST) {
    // A_e = c² (K1 ⊗ I + I ⊗ K1) + e_0 e_0^T is diagonal in the eigenbasis Q ⊗ Q of K1 (whose
    // first eigenvector is e_0 with λ_0 = 0): UT = Q [ (Q^T b Q) ∘ L ] Q^T, L = 1/(c²(λ_i+λ_j)), 1 at (0,0)
    const double ic2 = F.ic2e[e];
    // T1 = Q^T b into X1
#pragma unroll 1
    for (int c = 0; c < NU; ++c) {
      double t[NU];
#pragma unroll
      for (int i = 0; i < NU; ++i) t[i] = 0;
#pragma unroll
      for (int a = 0; a < NU; ++a) {
        const double x = bb(a, c);
#pragma unroll
        for (int i = 0; i < NU; ++i) t[i] = fma(B.Q[a][i], x, t[i]);
      }
#pragma unroll
      for (int i = 0; i < NU; ++i) X1(i, c) = t[i];
    }
    // T2 = (T1 Q) ∘ L into X2
#pragma unroll 1
    for (int i = 0; i < NU; ++i) {
      double t[NU];
#pragma unroll
      for (int jj = 0; jj < NU; ++jj) t[jj] = 0;
#pragma unroll
      for (int c = 0; c < NU; ++c) {
        const double x = X1(i, c);
#pragma unroll
        for (int jj = 0; jj < NU; ++jj) t[jj] = fma(x, B.Q[c][jj], t[jj]);
      }
#pragma unroll
      for (int jj = 0; jj < NU; ++jj) X2(i, jj) = (i == 0 && jj == 0) ? t[jj] : t[jj] * (B.ilam2[i][jj] * ic2);
    }
    // T3 = Q T2 into X1
#pragma unroll 1
    for (int jj = 0; jj < NU; ++jj) {
      double t[NU];
#pragma unroll
      for (int a = 0; a < NU; ++a) t[a] = 0;
#pragma unroll
      for (int i = 0; i < NU; ++i) {
        const double x = X2(i, jj);
#pragma unroll
        for (int a = 0; a < NU; ++a) t[a] = fma(B.Q[a][i], x, t[a]);
      }
#pragma unroll
      for (int a = 0; a < NU; ++a) X1(a, jj) = t[a];
    }
    // UT = T3 Q^T into X2, then back to X1
#pragma unroll 1
    for (int a = 0; a < NU; ++a) {
      double t[NU];
#pragma unroll
      for (int c = 0; c < NU; ++c) t[c] = 0;
#pragma unroll
      for (int jj = 0; jj < NU; ++jj) {
        const double x = X1(a, jj);
#pragma unroll
        for (int c = 0; c < NU; ++c) t[c] = fma(x, B.Q[c][jj], t[c]);
      }
#pragma unroll
      for (int c = 0; c < NU; ++c) X2(a, c) = t[c];
    }
#pragma unroll 1
    for (int a = 0; a < NU; ++a)
#pragma unroll
      for (int c = 0; c < NU; ++c) X1(a, c) = X2(a, c);
  } else {
    // packed upper triangle of the symmetric inverse, by columns: entry (i, j), i ≤ j, in row j(j+1)/2 + i
    constexpr int n = NU * NU;
    double *X = smem + tid, *bv = smem + NU * NU * BT + tid;   // X1 and b (= X2) as vectors a + NU c
#pragma unroll 1
    for (int i = 0; i < n; ++i) X[i * BT] = 0.0;
#pragma unroll 1
    for (int jj = 0; jj < n; ++jj) {
      const double bj = bv[jj * BT];
      const double *Ai = F.Ainv + (size_t)(jj * (jj + 1) / 2) * Eu + e;
      double s = 0;
#pragma unroll 4
      for (int i = 0; i < jj; ++i) {
        const double a = Ai[(size_t)i * Eu];
        X[i * BT] = fma(a, bj, X[i * BT]);
        s = fma(a, bv[i * BT], s);
      }
      X[jj * BT] = fma(Ai[(size_t)jj * Eu], bj, X[jj * BT] + s);
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
      if (S.mode == OUT_RHS) {
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

// ----------------------------------------------------------------------------
// k_mass: M(v_h) VT = R on every element (src/rhs.jl:778-951) and the v part of the outputs
// ----------------------------------------------------------------------------

// element of thread g: in the order of the Chebyshev step counts, or in mesh order
__device__ __forceinline__ int mass_element(const Fields &F, const StageIO &S, int g, int *pref) {
  if (!F.sorted) return g;
  int lo = 0;
#pragma unroll 1
  for (int b = NBIN - 1; b >= 0; --b)
    if (pref[b] <= g) { lo = b; break; }
  return F.bins[(size_t)lo * F.E + (g - pref[lo])];
}

template <int NU, int NV, bool CG>
__global__ void __launch_bounds__(MASS_THREADS)
    k_mass(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ Fields F,
           const __grid_constant__ StageIO S) {
  constexpr int QH = Basis<NU, NV>::QH, BT = MASS_THREADS;
  extern __shared__ double smem[];
  __shared__ int pref[NBIN];
  const int tid = threadIdx.x;
  const int E = F.E;
  const size_t Eu = (size_t)E;
  if (F.sorted) {
    // exclusive prefix sum of the counts of this stage's bins
    if (tid == 0) {
      int acc = 0;
      for (int b = 0; b < NBIN; ++b) { pref[b] = acc; acc += F.bin_count[S.parity * NBIN + b]; }
    }
    __syncthreads();
  }
  const int g = blockIdx.x * BT + tid;
  if (g >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int e = mass_element(F, S, g, pref);
  Blk<NV, BT> r{smem + tid}, X{smem + NV * NV * BT + tid};
  bool fin = true;

  // K P accumulated into O: O += P_h^T (G ∘ (P_h P P_h^T)) P_h, one row r2 of the point grid at a time
  auto addK = [&](Blk<NV, BT> P, Blk<NV, BT> O) {
#pragma unroll 1
    for (int r2 = 0; r2 < QH; ++r2) {
      double T[NV];
#pragma unroll
      for (int b = 0; b < NV; ++b) T[b] = 0.0;
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const double p = B.Ph[r2][a];
#pragma unroll
        for (int b = 0; b < NV; ++b) T[b] = fma(p, P(a, b), T[b]);
      }
      double Y[QH];
#pragma unroll
      for (int s2 = 0; s2 < QH; ++s2) Y[s2] = 0.0;
#pragma unroll
      for (int b = 0; b < NV; ++b)
#pragma unroll
        for (int s2 = 0; s2 < QH; ++s2) Y[s2] = fma(T[b], B.Ph[s2][b], Y[s2]);
#pragma unroll
      for (int s2 = 0; s2 < QH; ++s2) Y[s2] *= F.G[(r2 + QH * s2) * Eu + e];
      double Z[NV];
#pragma unroll
      for (int b = 0; b < NV; ++b) Z[b] = 0.0;
#pragma unroll
      for (int s2 = 0; s2 < QH; ++s2)
#pragma unroll
        for (int b = 0; b < NV; ++b) Z[b] = fma(Y[s2], B.Ph[s2][b], Z[b]);
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const double p = B.Ph[r2][a];
#pragma unroll
        for (int b = 0; b < NV; ++b) O(a, b) = fma(p, Z[b], O(a, b));
      }
    }
  };

  if constexpr (!CG) {
    // Chebyshev iteration (Saad Alg. 12.1, src/rhs.jl:921-939); K d is accumulated straight
    // into the residual after r -= d
    Blk<NV, BT> d{smem + 2 * NV * NV * BT + tid};
    const double th = F.th[e], de = F.de[e];
    const double s1 = th / de;
    const int n = F.cheb_common ? *F.nmax : F.nst[e];
    const double ith = 1.0 / th;
#pragma unroll 1
    for (int b = 0; b < NV; ++b)
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const double x = F.mrhs[(a + NV * b) * Eu + e];
        r(a, b) = x;
        d(a, b) = x * ith;
        X(a, b) = 0.0;
      }
    double rho = 1.0 / s1;
#pragma unroll 1
    for (int step = 1; step <= n; ++step) {
#pragma unroll 1
      for (int b = 0; b < NV; ++b)
#pragma unroll
        for (int a = 0; a < NV; ++a) {
          const double x = d(a, b);
          X(a, b) += x;
          r(a, b) -= x;
        }
      if (step == n) break;
      addK(d, r);
      const double rhon = 1.0 / (2.0 * s1 - rho);
      const double c1 = rhon * rho, c2 = 2.0 * rhon / de;
#pragma unroll 1
      for (int b = 0; b < NV; ++b)
#pragma unroll
        for (int a = 0; a < NV; ++a) d(a, b) = fma(c1, d(a, b), c2 * r(a, b));
      rho = rhon;
    }
  } else {
    // conjugate gradients from X = R (src/rhs.jl:824-853)
    Blk<NV, BT> p{smem + 2 * NV * NV * BT + tid}, Ap{smem + 3 * NV * NV * BT + tid};
    // G = 2βv_q W of this element
#pragma unroll 1
    for (int r2 = 0; r2 < QH; ++r2) {
      double T[NV];
#pragma unroll
      for (int b = 0; b < NV; ++b) T[b] = 0.0;
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const double pa = B.Ph[r2][a];
#pragma unroll
        for (int b = 0; b < NV; ++b) T[b] = fma(pa, S.xv[e + Eu * (a + NV * b)], T[b]);
      }
#pragma unroll
      for (int s2 = 0; s2 < QH; ++s2) {
        double gq = 0;
#pragma unroll
        for (int b = 0; b < NV; ++b) gq = fma(T[b], B.Ph[s2][b], gq);
        const size_t gi = (r2 + QH * s2) * Eu + e;
        F.G[gi] = 2.0 * F.beta[gi] * gq * B.Wh[r2][s2];
      }
    }
    double r0 = 0;
#pragma unroll 1
    for (int b = 0; b < NV; ++b)
#pragma unroll
      for (int a = 0; a < NV; ++a) {
        const double x = F.mrhs[(a + NV * b) * Eu + e];
        X(a, b) = x;
        p(a, b) = x;
        r(a, b) = 0.0;
        r0 = fma(x, x, r0);
      }
    addK(p, r);                                    // r = R - M X = K R for X = R
    double rr = 0;
#pragma unroll 1
    for (int b = 0; b < NV; ++b)
#pragma unroll
      for (int a = 0; a < NV; ++a) { const double x = r(a, b); p(a, b) = x; rr = fma(x, x, rr); }
    r0 = sqrt(r0);
    const int maxit = NV * NV + 10;
    int it = 0;
    bool bad = false;
    while (sqrt(rr) > F.mass_tol * r0 && it < maxit) {
      ++it;
#pragma unroll 1
      for (int b = 0; b < NV; ++b)
#pragma unroll
        for (int a = 0; a < NV; ++a) Ap(a, b) = 0.0;
      addK(p, Ap);
      double pAp = 0;
#pragma unroll 1
      for (int b = 0; b < NV; ++b)
#pragma unroll
        for (int a = 0; a < NV; ++a) { const double x = p(a, b) - Ap(a, b); Ap(a, b) = x; pAp = fma(p(a, b), x, pAp); }
      if (!(pAp > 0.0)) { bad = true; break; }
      const double al = rr / pAp;
      double rrn = 0;
#pragma unroll 1
      for (int b = 0; b < NV; ++b)
#pragma unroll
        for (int a = 0; a < NV; ++a) {
          X(a, b) = fma(al, p(a, b), X(a, b));
          const double x = fma(-al, Ap(a, b), r(a, b));
          r(a, b) = x;
          rrn = fma(x, x, rrn);
        }
      const double bt = rrn / rr;
#pragma unroll 1
      for (int b = 0; b < NV; ++b)
#pragma unroll
        for (int a = 0; a < NV; ++a) p(a, b) = fma(bt, p(a, b), r(a, b));
      rr = rrn;
    }
    if (bad) {
      atomicMin(F.err, (1ull << ERR_CLASS_SHIFT) | (unsigned long long)(e + 1));
      return;
    }
    if (sqrt(rr) > F.mass_tol * r0) atomicAdd(F.cg_nfail, 1u);
  }

  // ---- v outputs (RK4 as in k_stage)
#pragma unroll 1
  for (int b = 0; b < NV; ++b)
#pragma unroll
    for (int a = 0; a < NV; ++a) {
      const size_t l = e + Eu * (a + NV * b);
      const double kk = X(a, b);
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
  if (S.mode == OUT_RK4_LAST && !fin) atomicOr(F.nonfinite, 1u);
}

// shared memory of k_mass: r, X and d (Chebyshev); r, X, p and A p (CG)
__host__ __device__ constexpr size_t mass_smem(int nv, bool cg) {
  return (size_t)MASS_THREADS * (cg ? 4 : 3) * nv * nv * sizeof(double);
}

// Last RK4 update when the last stage may still raise an error inside k_mass
// (CG mode): u += (dt/6) acc unless an error was recorded.
__global__ void k_rk4_final(int n_u, int n_v, double *u, double *v, const double *accu, const double *accv,
                            double c, const unsigned long long *err, unsigned int *nonfinite);

// Device-side step bookkeeping after each RK4 step: counts completed steps and,
// when asked, stops the run after a non-finite result.
__global__ void k_step_done(unsigned long long *err, const unsigned int *nonfinite, int stop_nonfinite,
                            long long *steps_done);

}  // namespace wedg
