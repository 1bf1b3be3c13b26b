// Discrete adjoint of one right-hand side evaluation: given the state x = (U, V) and weights
// (λ_u, λ_v) of the outputs (ut, vt), the gradient Jᵀλ of λ_u·ut + λ_v·vt with respect to x.
//
// The forward evaluation (k_stage, k_cheb) is ut = A_e⁻¹ b, vt = M(v)⁻¹ R with
//   R = lifts of the flux slots A, D + volume terms of the v-equation + source,
//   b = -lifts of the slots F + volume terms of the u-equation + e₀ V₀₀,
// the slots affine in the traces of both elements of an interior face, nonlinear (through
// √(1 - kβv)) on absorbing boundary sides, and M(v) = I - K(v), K(v) = P_hᵀ diag(2βW v_q) P_h.
// Its transpose, in kernels:
//   μ = M(v)⁻¹ λ_v and ν = A_e⁻¹ λ_u        (k_cheb / k_cg and k_stage's u-solve: both symmetric)
//   the volume transposes                   (k_stage's volume terms on (-(h²/4) ν, μ): the
//                                            stiffness forms are symmetric)
//   k_adj_hats   the lift transposes: the weight of every flux slot at every side point
//   k_adj_mass   + P_hᵀ (2βW ∘ vt_q ∘ μ_q) P_h, the derivative of M(v) acting on vt
//   k_adj_face   the slots' derivatives with respect to the element's own traces (its own slots
//                and the neighbour's on the shared face), then the trace transposes.
// The slots of an interior face point are affine in its six traces and, on one-sided faces, the
// jump of the traces enters through the four one-sided coefficients only: their derivatives
// are closed forms in the face coefficients and the slot weights (face_weights below).
#pragma once

namespace wedg {

// Threads per block of the per-element adjoint kernels: long serial work per thread, so small
// blocks spread the elements of mid-size meshes over all SMs
constexpr int ADJ_THREADS = 32;

// Buffers of the adjoint kernels; every array in the state layout [e + E k] unless noted
struct AdjIO {
  const double *mu;      // μ = M⁻¹ λ_v (NV²)
  const double *nu;      // ν = A_e⁻¹ λ_u (NU²)
  double *nus;           // -(h²/4) ν, the u input of the volume transpose
  const double *vt;      // the forward vt at this state
  double *hat;           // slot weights, [((fam·4 + side)·NQ + i) E + e], fam A, D, F
  double *gu, *gv;       // the gradient; gu holds the volume's b on entry to k_adj_face
  const double *xv;      // the state's V (for the β-derivative of the mass matrix)
  double *gbe;           // per-element β-gradient that k_adj_mass adds to, or null
};

// One instance's arguments of a multi-instance adjoint launch (Multi<AdjArgs>): gc2, gal, gbe are
// k_adj_face's coefficient gradients (null unless PARAMS)
struct AdjArgs {
  Fields F;
  StageIO S;
  AdjIO A;
  double *gc2, *gal, *gbe;
};
using MultiAdj = Multi<AdjArgs, 28>;

// The weighted slot sums of an interior face point, from the scaled slot weights of the "+"
// element (hP: A, D, F) and of the "-" element (hM), with c² and α of both sides (a continuous
// face has c2m = c2p, afm = afp). With J, G, pen, sj of interior_flux,
//   Σ slots·weights = (pen sj - G)(hP_A - hM_A) + dvsp wP + dvsm wM,
//   wP = c2p hP_F - afp hP_D,  wM = afm hM_D - c2m hM_F,
//   dvsp = θ sj - τ J,  dvsm = -(1 - θ) sj - τ J,
// so a derivative of the sum is ∂(pen sj - G) wA - ∂J τ (wP + wM) plus the coefficients'
// direct terms.
struct FaceWeights {
  double wA, wP, wM, wS;  // wS = τ (wP + wM)
};
__device__ __forceinline__ FaceWeights face_weights(const Fields &F, const FaceCoef &c, double hPA, double hPD,
                                                    double hPF, double hMA, double hMD, double hMF) {
  FaceWeights w;
  w.wA = hPA - hMA;
  w.wP = c.c2p * hPF - c.afp * hPD;
  w.wM = c.afm * hMD - c.c2m * hMF;
  w.wS = F.tau * (w.wP + w.wM);
  return w;
}

// k_adj_hats: the weights of the slots A, D and F at every side point, the scaled traces of μ
// (values and derivatives) and of ν (derivatives) (src/rhs.jl:412-473 transposed:
// Â = (2/h) w_i tr_v(μ), D̂ = (4/h²) w_i tr_dv(μ), F̂ = -w_i tr_du(ν): the weights w_i folded
// into the values Pw, the sign of F̂ into the end vector E1F, the mesh factors applied to the
// traces); and nus.
template <int NU, int NV>
__device__ __forceinline__ void adj_hats_body(const Basis<NU, NV> &B, const Fields &F, const AdjIO &A, int e) {
  constexpr int NQ = NU;
  const int E = F.E;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const double s_nu = -1.0 / F.four_hh;
  {
    double M[NV][NV];
    load_regs<NV>(M, A.mu, E, e);
    trace4<NQ, NU, NV, false, true>(M, B.Pw, B.El, A.hat, 0, E, e, F.two_h);
    trace4<NQ, NU, NV, true, true>(M, B.Pw, B.E1l, A.hat, 1, E, e, F.four_hh);
  }
  double X[NU][NU];
  load_regs<NU>(X, A.nu, E, e);
  trace4<NQ, NU, NU, true>(X, B.Pw, B.E1F, A.hat, 2, E, e);
#pragma unroll
  for (int b = 0; b < NU; ++b)
#pragma unroll
    for (int a = 0; a < NU; ++a) A.nus[e + (size_t)E * (a + NU * b)] = s_nu * X[a][b];
}

template <int NU, int NV>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_hats(const __grid_constant__ Basis<NU, NV> B,
                                                   const __grid_constant__ Fields F, const AdjIO A) {
  adj_hats_body<NU, NV>(B, F, A, blockIdx.x * blockDim.x + threadIdx.x);
}

// tile = ADJ_THREADS elements per virtual block
template <int NU, int NV>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_hats_m(const __grid_constant__ Basis<NU, NV> B,
                                                     const __grid_constant__ MultiAdj P) {
  for (int vb = blockIdx.x; vb < P.first[P.n]; vb += gridDim.x) {
    const int inst = multi_begin(P, vb);
    adj_hats_body<NU, NV>(B, P.a[inst].F, P.a[inst].A, (vb - P.first[inst]) * P.tile + (int)threadIdx.x);
  }
}

// k_adj_mass: gv += P_hᵀ (2βW ∘ vt_q ∘ μ_q) P_h on every element, by the team layout of the mass
// solves: each unit forms the weights 2β vt_q of its two point rows (into G, which the forward
// solve of this state no longer needs) and applies them to μ with team_K. With A.gbe, also the
// β-derivative of μ·M(v) vt for β constant on the element, gbe[e] += Σ_q 2 W_q v_q vt_q μ_q.
template <int NU, int NV>
__device__ __forceinline__ void adj_mass_body(const Basis<NU, NV> &B, const Fields &F, const AdjIO &A, int e0) {
  using T = ChebTeam<NU, NV>;
  constexpr int QH = T::QH, U = T::U, NE = T::NE, J = T::J;
  __shared__ double sh[T::TPB * T::SLOT];
  __shared__ double Phs[QH * NV], PhWs[QH * NV];
  for (int i = threadIdx.x; i < QH * NV; i += blockDim.x) {
    Phs[i] = B.Ph[i / NV][i % NV];
    PhWs[i] = B.PhW[i / NV][i % NV];
  }
  __syncthreads();
  TeamPos tp;
  if (!team_pos<NU, NV>(tp)) return;
  const int e = e0 + tp.slot;
  if (e >= F.E) return;
  if (err_word(F) != ERR_NONE) return;
  const int u = tp.u;
  const unsigned tmask = tp.mask;
  const size_t Eu = (size_t)F.E;
  double *xs = sh + tp.slot * T::SLOT, *zs = xs + NE, *zd = zs + U * NV;
  double db = 0.0;                                      // Σ over the unit's points of w v_q vt_q μ_q
  {
    const int r1 = u, r2 = QH - 1 - u;
    auto tx = [&](int a, int b) { return A.vt[e + Eu * (a + NV * b)]; };
    double Tp[NV], Tm[NV];
    ph_row_pair<QH, NV>(B.Ph, r1, tx, Tp, Tm);
    auto gput = [&](const double (&Tv)[NV], int r, double (&Y)[QH]) {
      ph_to_points<QH, NV>(B.Ph, Tv, Y);
#pragma unroll
      for (int s2 = 0; s2 < QH; ++s2) {
        const size_t gi = (r + QH * s2) * Eu + e;
        F.G[gi] = Y[s2] * F.beta2[gi];
      }
    };
    double Yp[QH], Ym[QH];
    gput(Tp, r1, Yp);
    if (r2 != r1) gput(Tm, r2, Ym);
    if (A.gbe) {
      auto vx = [&](int a, int b) { return A.xv[e + Eu * (a + NV * b)]; };
      auto mx = [&](int a, int b) { return A.mu[e + Eu * (a + NV * b)]; };
      double Vp[NV], Vm[NV], Mp[NV], Mm[NV];
      ph_row_pair<QH, NV>(B.Ph, r1, vx, Vp, Vm);
      ph_row_pair<QH, NV>(B.Ph, r1, mx, Mp, Mm);
      auto row = [&](const double (&Y)[QH], const double (&Tv)[NV], const double (&Tmu)[NV]) {
        double Yv[QH], Yu[QH];
        ph_to_points<QH, NV>(B.Ph, Tv, Yv);
        ph_to_points<QH, NV>(B.Ph, Tmu, Yu);
        double r = 0.0;
#pragma unroll
        for (int s2 = 0; s2 < QH; ++s2) r = fma(B.wh[s2], Y[s2] * Yv[s2] * Yu[s2], r);
        return r;
      };
      db = B.wh[r1] * row(Yp, Vp, Mp);
      if (r2 != r1) db = fma(B.wh[r2], row(Ym, Vm, Mm), db);
    }
  }
  if (A.gbe) {
    db = team_sum<U>(db, tmask);
    if (u == 0) A.gbe[e] += 2.0 * db;
  }
  double acc[J];
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = u + U * j;
    acc[j] = 0.0;
    if (k < NE) {
      xs[k] = A.mu[e + Eu * k];
      acc[j] = A.gv[e + Eu * k];
    }
  }
  __syncwarp(tmask);
  team_K<NU, NV, 1>(B, F, Eu, e, u, tmask, Phs, PhWs, xs, zs, zd, acc);
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int k = u + U * j;
    if (k < NE) A.gv[e + Eu * k] = acc[j];
  }
}

template <int NU, int NV>
__global__ void __launch_bounds__(CHEB_THREADS, 3)
    k_adj_mass(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ Fields F, const AdjIO A) {
  adj_mass_body<NU, NV>(B, F, A, blockIdx.x * team_tile<NU, NV>());
}

// tile = team_tile elements per virtual block
template <int NU, int NV>
__global__ void __launch_bounds__(CHEB_THREADS, 3)
    k_adj_mass_m(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ MultiAdj P) {
  for (int vb = blockIdx.x; vb < P.first[P.n]; vb += gridDim.x) {
    const int inst = multi_begin(P, vb);
    adj_mass_body<NU, NV>(B, P.a[inst].F, P.a[inst].A, (vb - P.first[inst]) * P.tile);
  }
}

// The data of a physical side point (side_point's inputs): the coefficients there, the
// element's traces and the exact solution's data, with the outward sign sgn
struct SideData {
  double c2f, af, cf, bf, v_fp, gun, gvn, gu_ex, gv_ex, v_ex, sgn;
};
__device__ __forceinline__ SideData side_data(const Fields &F, const TimeF &tf, int s, int j, int k, int e, int i,
                                              int NQ) {
  const int N = F.N;
  const size_t Eu = (size_t)F.E;
  const int m = s < 2 ? k : j;
  SideData p;
  p.sgn = (s == 0 || s == 2) ? -1.0 : 1.0;
  size_t fi;
  const double *c2a, *afa, *cfa, *bfa;
  if (s < 2) { fi = (s == 0 ? 0 : N) + (size_t)(N + 1) * (k + (size_t)N * i); c2a = F.hc2; afa = F.haf; cfa = F.hcf; bfa = F.hbf; }
  else { fi = j + (size_t)N * ((s == 2 ? 0 : N) + (size_t)(N + 1) * i); c2a = F.vc2; afa = F.vaf; cfa = F.vcf; bfa = F.vbf; }
  p.c2f = c2a[fi]; p.af = afa[fi]; p.cf = cfa[fi]; p.bf = bfa[fi];
  const double *tr = F.tr;
  p.v_fp = tr[((1 * 4 + s) * NQ + i) * Eu + e];
  p.gun = p.sgn * (F.two_h * tr[((0 * 4 + s) * NQ + i) * Eu + e]);
  p.gvn = p.sgn * (F.two_h * tr[((2 * 4 + s) * NQ + i) * Eu + e]);
  const double spn = F.bspn[s][m + (size_t)N * i], sp = F.bsp[s][m + (size_t)N * i];
  p.gu_ex = p.sgn * (tf.ct * spn - spn);
  p.gv_ex = p.sgn * (-F.omega * tf.st * spn);
  p.v_ex = -F.omega * tf.st * sp;
  return p;
}

// Derivatives of the slots A, D, F of a physical side point with respect to the element's
// traces (du, v, dv) there (side_point's formulas differentiated), contracted with the slot
// weights h0, h1, h2: t[x] = Σ_q ∂q/∂x h_q.
__device__ __forceinline__ void boundary_trace_partials(const Fields &F, int s, const SideData &p, double h0,
                                                        double h1, double h2, double (&t)[3]) {
  const double sth = p.sgn * F.two_h;                  // d gun / d du = d gvn / d dv
  double dF1[3] = {0, 0, 0}, ddv[3] = {0, 0, 0};
  if (F.kind[s] == 3) {
    // wall: F1 = g2 (data), dv = -(κ/c)(c² gun + α gvn - g2)
    const double kc = -(F.kap[s] / p.cf);
    ddv[0] = kc * p.c2f * sth;
    ddv[2] = kc * p.af * sth;
  } else {
    const double g = F.gam[s], et = F.eta[s], sg = F.sig[s], kb = F.kb[s];
    const double sqf = sqrt(1.0 - kb * p.bf * p.v_fp);
    const double dsqf = -kb * p.bf / (2.0 * sqf);
    const double rho = et * (p.c2f * (p.gun - p.gu_ex) + p.af * (p.gvn - p.gv_ex)) +
                       g * p.cf * (sqf * p.v_fp - sqrt(1.0 - kb * p.bf * p.v_ex) * p.v_ex);
    const double drho[3] = {et * p.c2f * sth, g * p.cf * (sqf + p.v_fp * dsqf), et * p.af * sth};
    const double ke = -(g - sg * et) / p.cf;
    dF1[0] = p.c2f * sth - (et + sg * g) * drho[0];
    dF1[1] = -(et + sg * g) * drho[1];
    dF1[2] = p.af * sth - (et + sg * g) * drho[2];
    ddv[0] = ke * drho[0] / sqf;
    ddv[1] = ke * (drho[1] / sqf - rho * dsqf / (sqf * sqf));
    ddv[2] = ke * drho[2] / sqf;
  }
  // D = sgn α dv, F = -sgn c² dv
  const double m = p.sgn * (p.af * h1 - p.c2f * h2);
#pragma unroll
  for (int x = 0; x < 3; ++x) t[x] = fma(dF1[x], h0, ddv[x] * m);
}

// Derivatives of the weighted slots r = F1 h0 + q_D h1 + q_F h2 of a physical side point with
// respect to the coefficients c², α, c, β there (the traces and the data fixed): d[0..3]. With
// q_D = sgn α dv and q_F = -sgn c² dv, r = F1 h0 + dv · sgn (α h1 - c² h2).
__device__ __forceinline__ void boundary_coef_partials(const Fields &F, int s, const SideData &p, double h0,
                                                       double h1, double h2, double (&d)[4]) {
  const double c2f = p.c2f, af = p.af, cf = p.cf, bf = p.bf, sgn = p.sgn;
  double dF1[4], ddv[4], dv;
  if (F.kind[s] == 3) {
    // wall: F1 = c² gu_ex + α gv_ex, dv = -(κ/c)(c² (gun - gu_ex) + α (gvn - gv_ex))
    const double kc = F.kap[s] / cf, ru = p.gun - p.gu_ex, rv = p.gvn - p.gv_ex;
    const double rw = c2f * ru + af * rv;
    dv = -kc * rw;
    dF1[0] = p.gu_ex; dF1[1] = p.gv_ex; dF1[2] = 0.0; dF1[3] = 0.0;
    ddv[0] = -kc * ru; ddv[1] = -kc * rv; ddv[2] = kc * rw / cf; ddv[3] = 0.0;
  } else {
    // absorbing family: ρ = η (c² (gun - gu_ex) + α (gvn - gv_ex)) + γ c (√(1 - kβv) v - √(1 - kβv_ex) v_ex),
    // F1 = c² gun + α gvn - (η + σγ) ρ, dv = -(γ - ση) ρ / (c √(1 - kβv))
    const double g = F.gam[s], et = F.eta[s], sg = F.sig[s], kb = F.kb[s];
    const double sqf = sqrt(1.0 - kb * bf * p.v_fp), sqe = sqrt(1.0 - kb * bf * p.v_ex);
    const double dsqf = -kb * p.v_fp / (2.0 * sqf), dsqe = -kb * p.v_ex / (2.0 * sqe);   // ∂/∂β
    const double ru = p.gun - p.gu_ex, rv = p.gvn - p.gv_ex, rs = sqf * p.v_fp - sqe * p.v_ex;
    const double rho = et * (c2f * ru + af * rv) + g * cf * rs;
    const double drho[4] = {et * ru, et * rv, g * rs, g * cf * (p.v_fp * dsqf - p.v_ex * dsqe)};
    const double es = et + sg * g, kd = -(g - sg * et), den = cf * sqf;
    dF1[0] = p.gun - es * drho[0]; dF1[1] = p.gvn - es * drho[1]; dF1[2] = -es * drho[2]; dF1[3] = -es * drho[3];
    dv = kd * rho / den;
    ddv[0] = kd * drho[0] / den;
    ddv[1] = kd * drho[1] / den;
    ddv[2] = kd * (drho[2] / den - rho / (cf * den));
    ddv[3] = kd * (drho[3] / den - rho * dsqf / (sqf * den));
  }
  const double m = sgn * (af * h1 - c2f * h2);
  d[0] = fma(dF1[0], h0, fma(ddv[0], m, -sgn * dv * h2));
  d[1] = fma(dF1[1], h0, fma(ddv[1], m, sgn * dv * h1));
  d[2] = fma(dF1[2], h0, ddv[2] * m);
  d[3] = fma(dF1[3], h0, ddv[3] * m);
}

// k_adj_face: the trace weights of the element, t̂_x(s, i) = Σ_slots ∂slot/∂x · ŝlot over the
// element's own slots and (interior faces) the neighbour's slots of the shared point, for its
// traces x = du, v, dv; then the trace transposes (k_prep's trace4 transposed) into gu, gv. On
// entry gu holds the volume transpose's b; on exit gu, gv hold Jᵀλ.
//
// With PARAMS (the constant-coefficient kernels: c², α, β constant on each element), also the
// derivative of the stage's weighted output K̄·F(Y) with respect to the element's c² and α (and
// β through the faces), added to gc2[e], gal[e], gbe[e] (k_adj_mass adds the β-derivative of
// the mass matrix). With μ = M⁻¹K̄_v, ν = A_e⁻¹K̄_u and the forward ut at Y, K1 symmetric:
//   volume + u-solve   ∂/∂c² = <A1, V - ut> - (4/h²) <A2, U>,  ∂/∂α = -(4/h²) <A2, V>,
//                      A1 = K1 ν + ν K1,  A2 = K1 μ + μ K1
//                      (R ∋ -(4/h²)(c²(K1U + UK1) + α(K1V + VK1)), b ∋ c²(K1V + VK1),
//                       ∂A_e/∂c² ut = K1 ut + ut K1)
//   faces              the slots' derivatives times their weights: at an interior point of a
//                      one-sided face the element's own one-sided coefficients enter its own
//                      slots and the neighbour's; at a continuous face the shared face value
//                      enters the own slots (the neighbour adds its own); on a physical side
//                      c², α, c = √c², β enter the own slots.
//
// The points of a side come in mirrored pairs (i, NQ-1-i): the sums over the points are taken
// from their sums (even modes) and differences (odd modes), and the transposes of the two
// opposite sides (B and T, L and R) are applied together (Er = ±El, E1r = ∓E1l by mode parity).
template <int NU, int NV, bool PARAMS>
__device__ __forceinline__ void adj_face_body(const Basis<NU, NV> &B, const Fields &F, const StageIO &S,
                                              const AdjIO &A, double *gc2, double *gal, double *gbe, int e) {
  constexpr int NQ = NU;
  const int E = F.E, N = F.N;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int j = e % N, k = e / N;
  const size_t Eu = (size_t)E;
  const TimeF tf = time_factors(S);
  double dc2 = 0.0, dal = 0.0, dbe = 0.0;
  if constexpr (PARAMS) {
    // ---- volume and u-solve: ν and μ (padded to NU × NU) in registers, U, V, ut streamed
    double Nl[NU][NU], Ml[NU][NU];
#pragma unroll
    for (int b = 0; b < NU; ++b)
#pragma unroll
      for (int a = 0; a < NU; ++a) {
        Nl[a][b] = A.nu[e + Eu * (a + NU * b)];
        Ml[a][b] = (a < NV && b < NV) ? A.mu[e + Eu * (a + NV * b)] : 0.0;
      }
#pragma unroll
    for (int b = 0; b < NU; ++b)
#pragma unroll
      for (int a = 0; a < NU; ++a) {
        double a1 = 0.0, a2 = 0.0;
#pragma unroll
        for (int c = a & 1; c < NU; c += 2) {             // K1[a][c] = 0 for a + c odd
          a1 = fma(B.K1[a][c], Nl[c][b], a1);
          a2 = fma(B.K1[a][c], Ml[c][b], a2);
        }
#pragma unroll
        for (int c = b & 1; c < NU; c += 2) {
          a1 = fma(Nl[a][c], B.K1[c][b], a1);
          a2 = fma(Ml[a][c], B.K1[c][b], a2);
        }
        const size_t l = e + Eu * (a + NU * b);
        const double V = (a < NV && b < NV) ? S.xv[e + Eu * (a + NV * b)] : 0.0;
        dc2 = fma(a1, V - S.ut[l], fma(-F.four_hh * a2, S.xu[l], dc2));
        dal = fma(-F.four_hh * a2, V, dal);
      }
  }
  double gU[NU][NU], gV[NV][NV];
#pragma unroll
  for (int b = 0; b < NU; ++b)
#pragma unroll
    for (int a = 0; a < NU; ++a) gU[a][b] = -F.four_hh * A.gu[e + Eu * (a + NU * b)];
#pragma unroll
  for (int b = 0; b < NV; ++b)
#pragma unroll
    for (int a = 0; a < NV; ++a) gV[a][b] = A.gv[e + Eu * (a + NV * b)];
  gV[0][0] += A.nu[e];                                  // b[0][0] += V[0][0] transposed
  const double *tr = F.tr;
  auto T = [&](int fam, int side, int i, int el) { return tr[((fam * 4 + side) * NQ + i) * Eu + el]; };
  auto hat = [&](int fam, int side, int i, int el) { return A.hat[((fam * 4 + side) * NQ + i) * Eu + el]; };
  // t̂ (du, v, dv) at point i of side s, and the point's parameter terms
  auto point = [&](int s, bool boundary, int i, double (&t)[3]) {
    const double ho0 = hat(0, s, i, e), ho1 = hat(1, s, i, e), ho2 = hat(2, s, i, e);
    if (boundary) {
      const SideData p = side_data(F, tf, s, j, k, e, i, NQ);
      boundary_trace_partials(F, s, p, ho0, ho1, ho2, t);
      if constexpr (PARAMS) {
        double d[4];
        boundary_coef_partials(F, s, p, ho0, ho1, ho2, d);
        dc2 += d[0] + d[2] / (2.0 * p.cf);              // c = √c²
        dal += d[1];
        dbe += d[3];
      }
      return;
    }
    const bool plus = (s == 0 || s == 2);
    const int nb = s == 0 ? e - 1 : s == 1 ? e + 1 : s == 2 ? e - N : e + N;
    const int sn = s ^ 1;                               // the neighbour's side of this face
    size_t fi;
    const double *c2p_a, *afp_a, *c2m_a, *afm_a, *jc_a;
    if (s < 2) {
      fi = (s == 0 ? j : j + 1) + (size_t)(N + 1) * (k + (size_t)N * i);
      c2p_a = F.hc2; afp_a = F.haf; c2m_a = F.hc2m; afm_a = F.hafm; jc_a = F.hJC;
    } else {
      fi = j + (size_t)N * ((s == 2 ? k : k + 1) + (size_t)(N + 1) * i);
      c2p_a = F.vc2; afp_a = F.vaf; c2m_a = F.vc2m; afm_a = F.vafm; jc_a = F.vJC;
    }
    FaceCoef cf = face_coef(F, c2p_a, afp_a, c2m_a, afm_a, jc_a, fi);
    const bool os = F.one_sided;
    if (!os) { cf.c2m = cf.c2p; cf.afm = cf.afp; }
    const double hn0 = hat(0, sn, i, nb), hn1 = hat(1, sn, i, nb), hn2 = hat(2, sn, i, nb);
    const FaceWeights w = plus ? face_weights(F, cf, ho0, ho1, ho2, hn0, hn1, hn2)
                               : face_weights(F, cf, hn0, hn1, hn2, ho0, ho1, ho2);
    const double th = F.theta, a = F.two_h;
    const double pen = 0.5 * (cf.c2m + cf.c2p) * F.lu + 0.5 * (cf.afm + cf.afp) * F.lv;
    const double tv = pen * w.wA + th * w.wP - (1.0 - th) * w.wM;   // ∂/∂vm; ∂/∂vp = -tv
    // ∂/∂du of the own side: ∂J = ∓a c², ∂G = a θ c² (+) or a (1 - θ) c² (-); dv with α
    const double kd = plus ? w.wS - th * w.wA : -((1.0 - th) * w.wA + w.wS);
    t[0] = a * (plus ? cf.c2p : cf.c2m) * kd;
    t[1] = plus ? -tv : tv;
    t[2] = a * (plus ? cf.afp : cf.afm) * kd;
    if constexpr (PARAMS) {
      const int sm = s < 2 ? 1 : 3, spp = s < 2 ? 0 : 2;
      const int em = plus ? nb : e, ep = plus ? e : nb;
      const double vm = T(1, sm, i, em), vp = T(1, spp, i, ep);
      const double dum = T(0, sm, i, em), dup = T(0, spp, i, ep);
      const double dvm = T(2, sm, i, em), dvp = T(2, spp, i, ep);
      // the weights of both roles on one-sided faces, of the own role on continuous ones
      const FaceWeights wp = os ? w : plus ? face_weights(F, cf, ho0, ho1, ho2, 0.0, 0.0, 0.0)
                                           : face_weights(F, cf, 0.0, 0.0, 0.0, ho0, ho1, ho2);
      const double hP1 = plus ? ho1 : os ? hn1 : 0.0, hP2 = plus ? ho2 : os ? hn2 : 0.0;
      const double hM1 = plus ? (os ? hn1 : 0.0) : ho1, hM2 = plus ? (os ? hn2 : 0.0) : ho2;
      // which sides' coefficients are the element's: its own side (one-sided), both (continuous)
      const double dp = (!os || plus) ? 1.0 : 0.0, dm = (!os || !plus) ? 1.0 : 0.0;
      const double tau = F.tau;
      const double J = a * (cf.c2m * dum - cf.c2p * dup + cf.afm * dvm - cf.afp * dvp) + cf.K;
      const double sj = vm - vp;
      const double dvsp = th * sj - tau * J, dvsm = -(1.0 - th) * sj - tau * J;
      {
        const double dJ = a * (dm * dum - dp * dup), dG = a * ((1.0 - th) * dm * dum + th * dp * dup);
        const double dpen = 0.5 * (dm + dp) * F.lu;
        dc2 += (dpen * sj - dG) * wp.wA - dJ * wp.wS + dp * dvsp * hP2 - dm * dvsm * hM2;
      }
      {
        const double dJ = a * (dm * dvm - dp * dvp), dG = a * ((1.0 - th) * dm * dvm + th * dp * dvp);
        const double dpen = 0.5 * (dm + dp) * F.lv;
        dal += (dpen * sj - dG) * wp.wA - dJ * wp.wS - dp * dvsp * hP1 + dm * dvsm * hM1;
      }
    }
  };
  // sides in groups of NS: opposite sides together (B and T, then L and R) while the registers
  // allow, else one at a time
  constexpr int NS = NU <= 5 ? 2 : 1;
#pragma unroll 1
  for (int g0 = 0; g0 < 4; g0 += NS) {
    double qu[NS][NU], qv[NS][NV], qd[NS][NV];          // Σ_i P[i][b] t̂(s, i) per side and family
#pragma unroll
    for (int h = 0; h < NS; ++h) {
      const int s = g0 + h;
      const bool boundary = (s == 0 && j == 0) || (s == 1 && j == N - 1) || (s == 2 && k == 0) || (s == 3 && k == N - 1);
#pragma unroll
      for (int b = 0; b < NU; ++b) {
        qu[h][b] = 0.0;
        if (b < NV) { qv[h][b] = 0.0; qd[h][b] = 0.0; }
      }
#pragma unroll 1
      for (int i = 0; i < (NQ + 1) / 2; ++i) {
        double t1[3], t2[3];
        point(s, boundary, i, t1);
        const bool mid = 2 * i + 1 == NQ;               // the middle point: the odd modes vanish
        if (!mid) point(s, boundary, NQ - 1 - i, t2);
#pragma unroll
        for (int b = 0; b < NU; ++b) {
          const double p = B.P[i][b];
          const bool odd = b & 1;
          if (mid && odd) continue;
          const double su = mid ? t1[0] : odd ? t1[0] - t2[0] : t1[0] + t2[0];
          qu[h][b] = fma(p, su, qu[h][b]);
          if (b < NV) {
            const double sv = mid ? t1[1] : odd ? t1[1] - t2[1] : t1[1] + t2[1];
            const double sd = mid ? t1[2] : odd ? t1[2] - t2[2] : t1[2] + t2[2];
            qv[h][b] = fma(p, sv, qv[h][b]);
            qd[h][b] = fma(p, sd, qd[h][b]);
          }
        }
      }
    }
    // trace transposes: B/T contract the first index with the end values, L/R the second; the
    // far side's end vectors are Er[a] = (-1)^a El[a], E1r[a] = -(-1)^a E1l[a]
    const bool tb = g0 < 2;
    const bool right = NS == 1 && (g0 & 1);
#pragma unroll
    for (int a = 0; a < NU; ++a) {
      const bool odd = a & 1;
      const double e1 = B.E1l[a], e0 = B.El[a];
#pragma unroll
      for (int b = 0; b < NU; ++b) {
        double cu, cv = 0.0, cd = 0.0;
        if constexpr (NS == 2) {
          cu = odd ? qu[0][b] + qu[1][b] : qu[0][b] - qu[1][b];
          if (b < NV) {
            cv = odd ? qv[0][b] - qv[1][b] : qv[0][b] + qv[1][b];
            cd = odd ? qd[0][b] + qd[1][b] : qd[0][b] - qd[1][b];
          }
        } else {
          const double s1 = right ? (odd ? 1.0 : -1.0) : 1.0, s0 = right ? (odd ? -1.0 : 1.0) : 1.0;
          cu = s1 * qu[0][b];
          if (b < NV) {
            cv = s0 * qv[0][b];
            cd = s1 * qd[0][b];
          }
        }
        if (tb) gU[a][b] = fma(e1, cu, gU[a][b]);
        else gU[b][a] = fma(e1, cu, gU[b][a]);
        if (a < NV && b < NV) {
          if (tb) gV[a][b] = fma(e0, cv, fma(e1, cd, gV[a][b]));
          else gV[b][a] = fma(e0, cv, fma(e1, cd, gV[b][a]));
        }
      }
    }
  }
#pragma unroll
  for (int b = 0; b < NU; ++b)
#pragma unroll
    for (int a = 0; a < NU; ++a) A.gu[e + Eu * (a + NU * b)] = gU[a][b];
#pragma unroll
  for (int b = 0; b < NV; ++b)
#pragma unroll
    for (int a = 0; a < NV; ++a) A.gv[e + Eu * (a + NV * b)] = gV[a][b];
  if constexpr (PARAMS) {
    gc2[e] += dc2;
    gal[e] += dal;
    gbe[e] += dbe;
  }
}

template <int NU, int NV, bool PARAMS>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_face(const __grid_constant__ Basis<NU, NV> B,
                                                   const __grid_constant__ Fields F,
                                                   const __grid_constant__ StageIO S, const AdjIO A, double *gc2,
                                                   double *gal, double *gbe) {
  adj_face_body<NU, NV, PARAMS>(B, F, S, A, gc2, gal, gbe, blockIdx.x * blockDim.x + threadIdx.x);
}

// tile = ADJ_THREADS elements per virtual block
template <int NU, int NV, bool PARAMS>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_face_m(const __grid_constant__ Basis<NU, NV> B,
                                                     const __grid_constant__ MultiAdj P) {
  for (int vb = blockIdx.x; vb < P.first[P.n]; vb += gridDim.x) {
    const int inst = multi_begin(P, vb);
    const AdjArgs &a = P.a[inst];
    adj_face_body<NU, NV, PARAMS>(B, a.F, a.S, a.A, a.gc2, a.gal, a.gbe,
                                  (vb - P.first[inst]) * P.tile + (int)threadIdx.x);
  }
}

}  // namespace wedg
