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
  double *hat;           // slot weights, [((fam·4 + side)·NQ + i) E + e], fam A, D, F (unscaled)
  double *gu, *gv;       // the gradient; gu holds the volume's b on entry to k_adj_face
};

// k_adj_hats: the traces of μ (values and derivatives) and of ν (derivatives) on the four sides,
// whose scaled values are the weights of the slots A, D and F (src/rhs.jl:412-473 transposed:
// Â = (2/h) w_i tr_v(μ), D̂ = (4/h²) w_i tr_dv(μ), F̂ = -w_i tr_du(ν)); and nus.
template <int NU, int NV>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_hats(const __grid_constant__ Basis<NU, NV> B,
                                                   const __grid_constant__ Fields F, const AdjIO A) {
  constexpr int NQ = NU;
  const int E = F.E;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const double s_nu = -1.0 / F.four_hh;
  {
    double M[NV][NV];
    load_regs<NV>(M, A.mu, E, e);
    trace4<NQ, NU, NV, false>(M, B.P, B.El, A.hat, 0, E, e);
    trace4<NQ, NU, NV, true>(M, B.P, B.E1l, A.hat, 1, E, e);
  }
  double X[NU][NU];
  load_regs<NU>(X, A.nu, E, e);
  trace4<NQ, NU, NU, true>(X, B.P, B.E1l, A.hat, 2, E, e);
#pragma unroll
  for (int b = 0; b < NU; ++b)
#pragma unroll
    for (int a = 0; a < NU; ++a) A.nus[e + (size_t)E * (a + NU * b)] = s_nu * X[a][b];
}

// k_adj_mass: gv += P_hᵀ (2βW ∘ vt_q ∘ μ_q) P_h on every element, by the team layout of the mass
// solves: each unit forms the weights 2β vt_q of its two point rows (into G, which the forward
// solve of this state no longer needs) and applies them to μ with team_K.
template <int NU, int NV>
__global__ void __launch_bounds__(CHEB_THREADS, 3)
    k_adj_mass(const __grid_constant__ Basis<NU, NV> B, const __grid_constant__ Fields F, const AdjIO A) {
  using T = ChebTeam<NU, NV>;
  constexpr int QH = T::QH, U = T::U, NE = T::NE, J = T::J;
  __shared__ double sh[T::TPB * T::SLOT];
  __shared__ double Phs[QH * NV], PhWs[QH * NV];
  for (int i = threadIdx.x; i < QH * NV; i += CHEB_THREADS) {
    Phs[i] = B.Ph[i / NV][i % NV];
    PhWs[i] = B.PhW[i / NV][i % NV];
  }
  __syncthreads();
  TeamPos tp;
  if (!team_pos<NU, NV>(tp)) return;
  const int e = blockIdx.x * T::TPB + tp.slot;
  if (e >= F.E) return;
  if (err_word(F) != ERR_NONE) return;
  const int u = tp.u;
  const unsigned tmask = tp.mask;
  const size_t Eu = (size_t)F.E;
  double *xs = sh + tp.slot * T::SLOT, *zs = xs + NE, *zd = zs + U * NV;
  {
    const int r1 = u, r2 = QH - 1 - u;
    auto vx = [&](int a, int b) { return A.vt[e + Eu * (a + NV * b)]; };
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

// Partial derivatives of the slots A, D, F of a physical side point with respect to the
// element's traces (du, v, dv) there (the forward formulas of side_point, differentiated):
// d[q][x], q = A, D, F and x = du, v, dv.
template <int NU, int NV>
__device__ __forceinline__ void boundary_partials(const Fields &F, const TimeF &S, int s, int j, int k, int e,
                                                  int i, double (&d)[3][3]) {
  constexpr int NQ = NU;
  const int N = F.N;
  const double *tr = F.tr;
  const int m = s < 2 ? k : j;
  const double sgn = (s == 0 || s == 2) ? -1.0 : 1.0;
  size_t fi;
  const double *c2a, *afa, *cfa, *bfa;
  if (s < 2) { fi = (s == 0 ? 0 : N) + (size_t)(N + 1) * (k + (size_t)N * i); c2a = F.hc2; afa = F.haf; cfa = F.hcf; bfa = F.hbf; }
  else { fi = j + (size_t)N * ((s == 2 ? 0 : N) + (size_t)(N + 1) * i); c2a = F.vc2; afa = F.vaf; cfa = F.vcf; bfa = F.vbf; }
  const double c2f = c2a[fi], af = afa[fi], cf = cfa[fi];
  const double sth = sgn * F.two_h;                  // d gun / d du = d gvn / d dv
  double dF1[3] = {0, 0, 0}, ddv[3] = {0, 0, 0};
  if (F.kind[s] == 3) {
    // wall: F1 = g2 (data), dv = -(κ/c)(c² gun + α gvn - g2)
    const double kc = -(F.kap[s] / cf);
    ddv[0] = kc * c2f * sth;
    ddv[2] = kc * af * sth;
  } else {
    const double v_fp = tr[((1 * 4 + s) * NQ + i) * (size_t)F.E + e];
    const double gun = sgn * (F.two_h * tr[((0 * 4 + s) * NQ + i) * (size_t)F.E + e]);
    const double gvn = sgn * (F.two_h * tr[((2 * 4 + s) * NQ + i) * (size_t)F.E + e]);
    const double spn = F.bspn[s][m + (size_t)N * i], sp = F.bsp[s][m + (size_t)N * i];
    const double gu_ex = sgn * (S.ct * spn - spn);
    const double gv_ex = sgn * (-F.omega * S.st * spn);
    const double v_ex = -F.omega * S.st * sp;
    const double bf = bfa[fi];
    const double g = F.gam[s], et = F.eta[s], sg = F.sig[s], kb = F.kb[s];
    const double sqf = sqrt(1.0 - kb * bf * v_fp);
    const double dsqf = -kb * bf / (2.0 * sqf);
    const double rho_num = et * (c2f * gun + af * gvn) + g * cf * sqf * v_fp;
    const double rho_ex = et * (c2f * gu_ex + af * gv_ex) + g * cf * sqrt(1.0 - kb * bf * v_ex) * v_ex;
    const double rho = rho_num - rho_ex;
    const double drho[3] = {et * c2f * sth, g * cf * (sqf + v_fp * dsqf), et * af * sth};
    const double ke = -(g - sg * et) / cf;
    dF1[0] = c2f * sth - (et + sg * g) * drho[0];
    dF1[1] = -(et + sg * g) * drho[1];
    dF1[2] = af * sth - (et + sg * g) * drho[2];
    ddv[0] = ke * drho[0] / sqf;
    ddv[1] = ke * (drho[1] / sqf - rho * dsqf / (sqf * sqf));
    ddv[2] = ke * drho[2] / sqf;
  }
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    d[0][x] = dF1[x];
    d[1][x] = sgn * (af * ddv[x]);
    d[2][x] = -sgn * (c2f * ddv[x]);
  }
}

// k_adj_face: the trace weights of the element, t̂_x(s, i) = Σ_slots ∂slot/∂x · ŝlot over the
// element's own slots and (interior faces) the neighbour's slots of the shared point, for its
// traces x = du, v, dv; then the trace transposes (k_prep's trace4 transposed) into gu, gv.
// The interior slots are affine in the six traces of the face point (interior_flux), so their
// derivatives are read off exactly from the values at zero and at unit traces.
// On entry gu holds the volume transpose's b; on exit gu, gv hold Jᵀλ.
template <int NU, int NV>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_face(const __grid_constant__ Basis<NU, NV> B,
                                                   const __grid_constant__ Fields F,
                                                   const __grid_constant__ StageIO S, const AdjIO A) {
  constexpr int NQ = NU;
  const int E = F.E, N = F.N;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int j = e % N, k = e / N;
  const size_t Eu = (size_t)E;
  const TimeF tf = time_factors(S);
  auto hat = [&](int fam, int side, int i, int el) {
    const double h = A.hat[((fam * 4 + side) * NQ + i) * Eu + el];
    const double w = B.w[i];
    return fam == 0 ? F.two_h * w * h : fam == 1 ? F.four_hh * w * h : -w * h;
  };
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
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    const bool boundary = (s == 0 && j == 0) || (s == 1 && j == N - 1) || (s == 2 && k == 0) || (s == 3 && k == N - 1);
    double qu[NU], qv[NV], qd[NV];                      // Σ_i P[i][b] t̂(s, i) per trace family
#pragma unroll
    for (int b = 0; b < NU; ++b) {
      qu[b] = 0.0;
      if (b < NV) { qv[b] = 0.0; qd[b] = 0.0; }
    }
#pragma unroll 1
    for (int i = 0; i < NQ; ++i) {
      double t[3] = {0.0, 0.0, 0.0};                    // t̂ for du, v, dv
      if (boundary) {
        double d[3][3];
        boundary_partials<NU, NV>(F, tf, s, j, k, e, i, d);
        const double h3[3] = {hat(0, s, i, e), hat(1, s, i, e), hat(2, s, i, e)};
#pragma unroll
        for (int x = 0; x < 3; ++x) t[x] = d[0][x] * h3[0] + d[1][x] * h3[1] + d[2][x] * h3[2];
      } else {
        const bool plus = (s == 0 || s == 2);
        const int nb = s == 0 ? e - 1 : s == 1 ? e + 1 : s == 2 ? e - N : e + N;
        const int sn = s ^ 1;                           // the neighbour's side of this face
        size_t fi;
        const double *c2p_a, *afp_a, *c2m_a, *afm_a, *jc_a;
        if (s < 2) {
          fi = (s == 0 ? j : j + 1) + (size_t)(N + 1) * (k + (size_t)N * i);
          c2p_a = F.hc2; afp_a = F.haf; c2m_a = F.hc2m; afm_a = F.hafm; jc_a = F.hJC;
        } else {
          fi = j + (size_t)N * ((s == 2 ? k : k + 1) + (size_t)(N + 1) * i);
          c2p_a = F.vc2; afp_a = F.vaf; c2m_a = F.vc2m; afm_a = F.vafm; jc_a = F.vJC;
        }
        const FaceCoef cf = face_coef(F, c2p_a, afp_a, c2m_a, afm_a, jc_a, fi);
        const double ho[3] = {hat(0, s, i, e), hat(1, s, i, e), hat(2, s, i, e)};
        const double hn[3] = {hat(0, sn, i, nb), hat(1, sn, i, nb), hat(2, sn, i, nb)};
        // own traces in the order (dum, dup, vm, vp, dvm, dvp): du, v, dv of the own side
        const int own[3] = {plus ? 1 : 0, plus ? 3 : 2, plus ? 5 : 4};
        double z[3][2];                                 // slots at zero traces: own role, neighbour role
        interior_flux(F, cf, plus, 0, 0, 0, 0, 0, 0, z[0][0], z[1][0], z[2][0]);
        interior_flux(F, cf, !plus, 0, 0, 0, 0, 0, 0, z[0][1], z[1][1], z[2][1]);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          double in[6] = {0, 0, 0, 0, 0, 0};
          in[own[x]] = 1.0;
          double Ao, Do, Fo, An, Dn, Fn;
          interior_flux(F, cf, plus, in[0], in[1], in[2], in[3], in[4], in[5], Ao, Do, Fo);
          interior_flux(F, cf, !plus, in[0], in[1], in[2], in[3], in[4], in[5], An, Dn, Fn);
          t[x] = (Ao - z[0][0]) * ho[0] + (Do - z[1][0]) * ho[1] + (Fo - z[2][0]) * ho[2] +
                 (An - z[0][1]) * hn[0] + (Dn - z[1][1]) * hn[1] + (Fn - z[2][1]) * hn[2];
        }
      }
#pragma unroll
      for (int b = 0; b < NU; ++b) {
        const double p = B.P[i][b];
        qu[b] = fma(p, t[0], qu[b]);
        if (b < NV) {
          qv[b] = fma(p, t[1], qv[b]);
          qd[b] = fma(p, t[2], qd[b]);
        }
      }
    }
    // trace transposes: B/T sides contract the first index with the end values, L/R the second
    const bool right = (s == 1 || s == 3);
#pragma unroll
    for (int a = 0; a < NU; ++a) {
      const double sa = (a & 1) && right ? -1.0 : 1.0;  // Er = ±El, E1r = ∓E1l by mode parity
      const double e1 = right ? -sa * B.E1l[a] : B.E1l[a];
      const double e0 = right ? sa * B.El[a] : B.El[a];
#pragma unroll
      for (int b = 0; b < NU; ++b) {
        if (s < 2) {
          gU[a][b] = fma(e1, qu[b], gU[a][b]);
          if (a < NV && b < NV) gV[a][b] = fma(e0, qv[b], fma(e1, qd[b], gV[a][b]));
        } else {
          gU[b][a] = fma(e1, qu[b], gU[b][a]);
          if (a < NV && b < NV) gV[b][a] = fma(e0, qv[b], fma(e1, qd[b], gV[b][a]));
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
}

// The slots of a physical side point as functions of the coefficients there (side_point's
// formulas with c², α, c, β as arguments), for their derivatives in k_adj_param
__device__ __forceinline__ void boundary_slots(const Fields &F, int s, double c2f, double af, double cf, double bf,
                                               double v_fp, double gun, double gvn, double gu_ex, double gv_ex,
                                               double v_ex, double sgn, double (&q)[3]) {
  double F1, dv;
  if (F.kind[s] == 3) {
    const double g2 = c2f * gu_ex + af * gv_ex;
    const double rho_w = c2f * gun + af * gvn - g2;
    dv = -(F.kap[s] / cf) * rho_w;
    F1 = g2;
  } else {
    const double g = F.gam[s], et = F.eta[s], sg = F.sig[s], kb = F.kb[s];
    const double sqf = sqrt(1.0 - kb * bf * v_fp);
    const double rho_num = et * (c2f * gun + af * gvn) + g * cf * sqf * v_fp;
    const double rho_ex = et * (c2f * gu_ex + af * gv_ex) + g * cf * sqrt(1.0 - kb * bf * v_ex) * v_ex;
    const double rho = rho_num - rho_ex;
    F1 = c2f * gun + af * gvn - (et + sg * g) * rho;
    dv = -(g - sg * et) / (cf * sqf) * rho;
  }
  q[0] = F1;
  q[1] = sgn * (af * dv);
  q[2] = -sgn * (c2f * dv);
}

// k_adj_param: for the constant-coefficient kernels (c², α, β constant on each element), the
// derivative of the stage's weighted output K̄·F(Y) with respect to the element's c², α and β,
// added to gc2[e], gal[e], gbe[e]. With μ = M⁻¹K̄_v, ν = A_e⁻¹K̄_u and the forward outputs ut, vt
// at Y (all from the adjoint evaluation just made at Y):
//   volume   μ·∂R/∂p + ν·∂b/∂p   (R ∋ -(4/h²)(c²(K1U + UK1) + α(K1V + VK1)), b ∋ c²(K1V + VK1))
//   u-solve  -ν·(∂A_e/∂c²) ut = -ν·(K1 ut + ut K1)
//   mass     μ·(∂K/∂β) vt = Σ_points 2 W v_q vt_q μ_q
//   faces    the slots' derivatives times their weights (the hats): at an interior point of a
//            one-sided face, the element's own coefficient enters its own slots and the
//            neighbour's (each slot is quadratic in one coefficient, so a central difference
//            of step |c| is exact); at a continuous face the shared face value enters the own
//            slots (the neighbour adds its own); on a physical side c², α, c = √c², β enter the
//            own slots (central differences of relative step 1e-6).
template <int NU, int NV>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_param(const __grid_constant__ Basis<NU, NV> B,
                                                    const __grid_constant__ Fields F,
                                                    const __grid_constant__ StageIO S, const AdjIO A,
                                                    double *gc2, double *gal, double *gbe) {
  constexpr int NQ = NU, QH = Basis<NU, NV>::QH;
  const int E = F.E, N = F.N;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  if (err_word(F) != ERR_NONE) return;
  const int j = e % N, k = e / N;
  const size_t Eu = (size_t)E;
  const TimeF tf = time_factors(S);
  double dc2 = 0.0, dal = 0.0, dbe = 0.0;
  // ---- volume and u-solve: the element's blocks loaded once (V and μ padded to NU × NU)
  {
    double Ul[NU][NU], Vl[NU][NU], Ml[NU][NU], Nl[NU][NU], Tl[NU][NU];
#pragma unroll
    for (int b = 0; b < NU; ++b)
#pragma unroll
      for (int a = 0; a < NU; ++a) {
        const size_t lu = e + Eu * (a + NU * b), lv = e + Eu * (a + NV * b);
        const bool inv = a < NV && b < NV;
        Ul[a][b] = S.xu[lu];
        Nl[a][b] = A.nu[lu];
        Tl[a][b] = S.ut[lu];
        Vl[a][b] = inv ? S.xv[lv] : 0.0;
        Ml[a][b] = inv ? A.mu[lv] : 0.0;
      }
#pragma unroll 1
    for (int a = 0; a < NU; ++a)
#pragma unroll
      for (int b = 0; b < NU; ++b) {
        double ku = 0, kv = 0, kt = 0;
#pragma unroll
        for (int c = 0; c < NU; ++c) {
          const double l = B.K1[a][c], r = B.K1[c][b];
          ku = fma(l, Ul[c][b], fma(Ul[a][c], r, ku));
          kv = fma(l, Vl[c][b], fma(Vl[a][c], r, kv));
          kt = fma(l, Tl[c][b], fma(Tl[a][c], r, kt));
        }
        const double m = Ml[a][b], n = Nl[a][b];
        dc2 += -F.four_hh * m * ku - n * kt + n * kv;   // R (v-block: μ is zero outside), u-solve, b
        dal += -F.four_hh * m * kv;
      }
  }
  // ---- mass: Σ_points 2 W v_q vt_q μ_q (β constant on the element)
  {
    double Tv[QH][NV], Tt[QH][NV], Tm[QH][NV];
    for (int r = 0; r < QH; ++r)
      for (int b = 0; b < NV; ++b) {
        double x = 0, y = 0, z = 0;
        for (int a = 0; a < NV; ++a) {
          x += B.Ph[r][a] * S.xv[e + Eu * (a + NV * b)];
          y += B.Ph[r][a] * S.vt[e + Eu * (a + NV * b)];
          z += B.Ph[r][a] * A.mu[e + Eu * (a + NV * b)];
        }
        Tv[r][b] = x; Tt[r][b] = y; Tm[r][b] = z;
      }
    for (int r = 0; r < QH; ++r)
      for (int s2 = 0; s2 < QH; ++s2) {
        double x = 0, y = 0, z = 0;
        for (int b = 0; b < NV; ++b) { x += Tv[r][b] * B.Ph[s2][b]; y += Tt[r][b] * B.Ph[s2][b]; z += Tm[r][b] * B.Ph[s2][b]; }
        dbe += 2.0 * (B.PhW[r][0] / B.Ph[r][0]) * (B.PhW[s2][0] / B.Ph[s2][0]) * x * y * z;
      }
  }
  // ---- faces
  const double *tr = F.tr;
  auto T = [&](int fam, int side, int i, int el) { return tr[((fam * 4 + side) * NQ + i) * Eu + el]; };
  auto hat = [&](int fam, int side, int i, int el) {
    const double h = A.hat[((fam * 4 + side) * NQ + i) * Eu + el];
    const double w = B.w[i];
    return fam == 0 ? F.two_h * w * h : fam == 1 ? F.four_hh * w * h : -w * h;
  };
  for (int s = 0; s < 4; ++s) {
    const bool boundary = (s == 0 && j == 0) || (s == 1 && j == N - 1) || (s == 2 && k == 0) || (s == 3 && k == N - 1);
    for (int i = 0; i < NQ; ++i) {
      const double ho[3] = {hat(0, s, i, e), hat(1, s, i, e), hat(2, s, i, e)};
      if (boundary) {
        const int m = s < 2 ? k : j;
        const double sgn = (s == 0 || s == 2) ? -1.0 : 1.0;
        size_t fi;
        const double *c2a, *afa, *cfa, *bfa;
        if (s < 2) { fi = (s == 0 ? 0 : N) + (size_t)(N + 1) * (k + (size_t)N * i); c2a = F.hc2; afa = F.haf; cfa = F.hcf; bfa = F.hbf; }
        else { fi = j + (size_t)N * ((s == 2 ? 0 : N) + (size_t)(N + 1) * i); c2a = F.vc2; afa = F.vaf; cfa = F.vcf; bfa = F.vbf; }
        const double c2f = c2a[fi], af = afa[fi], cf = cfa[fi], bf = bfa[fi];
        const double v_fp = T(1, s, i, e);
        const double gun = sgn * (F.two_h * T(0, s, i, e)), gvn = sgn * (F.two_h * T(2, s, i, e));
        const double spn = F.bspn[s][m + (size_t)N * i], sp = F.bsp[s][m + (size_t)N * i];
        const double gu_ex = sgn * (tf.ct * spn - spn), gv_ex = sgn * (-F.omega * tf.st * spn);
        const double v_ex = -F.omega * tf.st * sp;
        double x[4] = {c2f, af, cf, bf}, d[4];
        for (int p = 0; p < 4; ++p) {
          const double hstep = 1e-6 * (fabs(x[p]) > 1e-300 ? fabs(x[p]) : 1.0);
          double qp[3], qm[3], y[4] = {x[0], x[1], x[2], x[3]};
          y[p] = x[p] + hstep;
          boundary_slots(F, s, y[0], y[1], y[2], y[3], v_fp, gun, gvn, gu_ex, gv_ex, v_ex, sgn, qp);
          y[p] = x[p] - hstep;
          boundary_slots(F, s, y[0], y[1], y[2], y[3], v_fp, gun, gvn, gu_ex, gv_ex, v_ex, sgn, qm);
          d[p] = ((qp[0] - qm[0]) * ho[0] + (qp[1] - qm[1]) * ho[1] + (qp[2] - qm[2]) * ho[2]) / (2.0 * hstep);
        }
        dc2 += d[0] + d[2] / (2.0 * cf);        // c = √c²
        dal += d[1];
        dbe += d[3];
      } else {
        const bool plus = (s == 0 || s == 2);
        const int nb = s == 0 ? e - 1 : s == 1 ? e + 1 : s == 2 ? e - N : e + N;
        const int sn = s ^ 1;
        const int sm = s < 2 ? 1 : 3, spp = s < 2 ? 0 : 2;
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
        const FaceCoef cf = face_coef(F, c2p_a, afp_a, c2m_a, afm_a, jc_a, fi);
        const double vm = T(1, sm, i, em), vp = T(1, spp, i, ep);
        const double dum = T(0, sm, i, em), dup = T(0, spp, i, ep);
        const double dvm = T(2, sm, i, em), dvp = T(2, spp, i, ep);
        const double hn[3] = {hat(0, sn, i, nb), hat(1, sn, i, nb), hat(2, sn, i, nb)};
        // weighted slots (own, and with the neighbour's role and weights on one-sided faces)
        auto wslots = [&](const FaceCoef &c) {
          double Ao, Do, Fo;
          interior_flux(F, c, plus, dum, dup, vm, vp, dvm, dvp, Ao, Do, Fo);
          double r = Ao * ho[0] + Do * ho[1] + Fo * ho[2];
          if (F.one_sided) {
            double An, Dn, Fn;
            interior_flux(F, c, !plus, dum, dup, vm, vp, dvm, dvp, An, Dn, Fn);
            r += An * hn[0] + Dn * hn[1] + Fn * hn[2];
          }
          return r;
        };
        // the element's own coefficient: its side's values on one-sided faces, the face value else
        for (int p = 0; p < 2; ++p) {
          FaceCoef cp = cf, cm = cf;
          double *xp, *xm, x;
          if (F.one_sided && !plus) { xp = p ? &cp.afm : &cp.c2m; xm = p ? &cm.afm : &cm.c2m; x = p ? cf.afm : cf.c2m; }
          else { xp = p ? &cp.afp : &cp.c2p; xm = p ? &cm.afp : &cm.c2p; x = p ? cf.afp : cf.c2p; }
          const double hstep = fabs(x) > 1e-300 ? fabs(x) : 1.0;
          *xp = x + hstep;
          *xm = x - hstep;
          const double d = (wslots(cp) - wslots(cm)) / (2.0 * hstep);
          if (p == 0) dc2 += d;
          else dal += d;
        }
      }
    }
  }
  gc2[e] += dc2;
  gal[e] += dal;
  gbe[e] += dbe;
}

}  // namespace wedg
