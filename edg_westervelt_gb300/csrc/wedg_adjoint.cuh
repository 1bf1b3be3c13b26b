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
__global__ void __launch_bounds__(128) k_adj_hats(const __grid_constant__ Basis<NU, NV> B,
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
__global__ void __launch_bounds__(128) k_adj_face(const __grid_constant__ Basis<NU, NV> B,
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

}  // namespace wedg
