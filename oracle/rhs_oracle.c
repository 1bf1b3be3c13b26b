/*
 * CPU oracle of the WesterveltEDG.jl right-hand side and RK4 step.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/ as the checker and by bench.py as
 * the timed CPU port of the reference. Never linked into the product.
 *
 * Restates src/rhs.jl (v0.3.0) of the reference, function by function:
 *   traces        _trace4! / _traces!             rhs.jl:384-410, 573-580
 *   faces         _interior_faces! / _os!         rhs.jl:589-700
 *   boundary      _boundary_side! / _abc_face /   rhs.jl:65-128, 702-776
 *                 _wall_face / _boundary_key
 *   volume        _volume_terms!                  rhs.jl:309-333
 *   source        _scale_source!                  rhs.jl:335-350
 *   lifts         _lifts!                         rhs.jl:412-473
 *   u-equation    _u_equation!                    rhs.jl:352-382
 *   Chebyshev     _cheb_setup! / _cheb_steps /    rhs.jl:870-951
 *                 _cheb_iterate!
 *   CG            _mass_cg_block!                 rhs.jl:821-853
 *   RK4           rk4_step! / _rk4_stage! /       solver.jl:278-321
 *                 _rk4_final!
 * Arrays use the reference's column-major layouts (see oracle/precompute.py).
 * All elements take the global maximum Chebyshev step count, as the reference
 * does. Element work runs on OpenMP threads; results do not depend on the
 * thread count.
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int N, nu, nv, qh;
  double theta, tau, lu, lv, omega;
  int mms_on, src_on, one_sided, cheb;
  double mass_tol, src_omega, src_Ts;
  int kind[4]; /* per side bot, top, lft, rgt: 0 absorbing_2beta, 1 absorbing, 2 dirichlet, 3 wall */
  double gam[4], eta[4], sig[4], kb[4], kap[4];
  const double *w, *P_u, *S_u, *Ebl_u, *Ebr_u, *E1bl_u, *E1br_u;
  const double *P_h, *W_h;
  const double *Cw, *Aw, *Ainv;
  const double *hc2, *haf, *hcf, *hbf, *vc2, *vaf, *vcf, *vbf;
  const double *hc2m, *hafm, *vc2m, *vafm, *hJC, *vJC;
  const double *bcB_sp, *bcB_spy, *bcT_sp, *bcT_spy, *bcL_sp, *bcL_spx, *bcR_sp, *bcR_spx;
  const double *PiSP, *PiBSP2, *PiCdiv, *PiDdiv, *src_projE;
  const double *beta_hq, *beta_hE;
} or_pre;

typedef struct {
  or_pre p;
  double *tr[12];   /* duB duT duL duR vB vT vL vR dvB dvT dvL dvR, (nq,N,N) */
  double *sl[12];   /* AB AT AL AR DB DT DL DR FB FT FL FR, (nq,N,N) */
  double *Rv, *VB, *Fu, *UT, *VT; /* element-last */
  double *th, *de, *s1, *G;       /* Chebyshev interval data and G = 2βv_q W */
  int *nst;                       /* per-element step counts */
  double *k[4][2], *su, *sv;
} or_ws;

enum { T_DU = 0, T_V = 4, T_DV = 8 };
enum { S_A = 0, S_D = 4, S_F = 8 };
enum { SB = 0, ST = 1, SL = 2, SR = 3 };

or_ws *or_create(const or_pre *p) {
  or_ws *ws = (or_ws *)calloc(1, sizeof(or_ws));
  ws->p = *p;
  size_t E = (size_t)p->N * p->N, nq = p->nu;
  for (int i = 0; i < 12; ++i) {
    ws->tr[i] = (double *)calloc(nq * E, sizeof(double));
    ws->sl[i] = (double *)calloc(nq * E, sizeof(double));
  }
  size_t nu2 = (size_t)p->nu * p->nu, nv2 = (size_t)p->nv * p->nv;
  ws->Rv = (double *)calloc(nv2 * E, sizeof(double));
  ws->VT = (double *)calloc(nv2 * E, sizeof(double));
  ws->VB = (double *)calloc(nu2 * E, sizeof(double));
  ws->Fu = (double *)calloc(nu2 * E, sizeof(double));
  ws->UT = (double *)calloc(nu2 * E, sizeof(double));
  ws->th = (double *)calloc(E, sizeof(double));
  ws->de = (double *)calloc(E, sizeof(double));
  ws->s1 = (double *)calloc(E, sizeof(double));
  ws->G = (double *)calloc((size_t)p->qh * p->qh * E, sizeof(double));
  ws->nst = (int *)calloc(E, sizeof(int));
  for (int s = 0; s < 4; ++s) {
    ws->k[s][0] = (double *)calloc(nu2 * E, sizeof(double));
    ws->k[s][1] = (double *)calloc(nv2 * E, sizeof(double));
  }
  ws->su = (double *)calloc(nu2 * E, sizeof(double));
  ws->sv = (double *)calloc(nv2 * E, sizeof(double));
  return ws;
}

void or_destroy(or_ws *ws) {
  if (!ws) return;
  for (int i = 0; i < 12; ++i) { free(ws->tr[i]); free(ws->sl[i]); }
  free(ws->Rv); free(ws->VT); free(ws->VB); free(ws->Fu); free(ws->UT);
  free(ws->th); free(ws->de); free(ws->s1); free(ws->G); free(ws->nst);
  for (int s = 0; s < 4; ++s) { free(ws->k[s][0]); free(ws->k[s][1]); }
  free(ws->su); free(ws->sv);
  free(ws);
}

/* element e's modal block of a state array x (layout (N,N,n,n)) */
static void load_elem(double *X, const double *x, size_t e, size_t E, int n) {
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) X[a + n * b] = x[e + E * (a + (size_t)n * b)];
}

/* _trace4!: oB[i] = Σ_b P[i,b] Σ_a El[a] X[a,b]; oL, oR contract the x-mode (rhs.jl:388-410) */
static void trace4(double *oB, double *oT, double *oL, double *oR, const double *P, int nq, int n,
                   const double *El, const double *Er, const double *X) {
  for (int i = 0; i < nq; ++i) oB[i] = oT[i] = oL[i] = oR[i] = 0.0;
  for (int b = 0; b < n; ++b) {
    double sB = 0, sT = 0, sL = 0, sR = 0;
    for (int a = 0; a < n; ++a) {
      double x = X[a + n * b], xt = X[b + n * a];
      sB += El[a] * x; sT += Er[a] * x; sL += El[a] * xt; sR += Er[a] * xt;
    }
    for (int i = 0; i < nq; ++i) {
      double pp = P[i + nq * b];
      oB[i] += pp * sB; oT[i] += pp * sT; oL[i] += pp * sL; oR[i] += pp * sR;
    }
  }
}

/* out (m x m) = L (m x n) Z (n x n) R^T, L and R column-major with leading dimension ldl/ldr */
static void contract_fwd(double *out, const double *L, int ldl, const double *R, int ldr, const double *Z,
                         int m, int n) {
  double T[16 * 16];
  for (int b = 0; b < n; ++b)
    for (int r = 0; r < m; ++r) {
      double s = 0;
      for (int a = 0; a < n; ++a) s += L[r + ldl * a] * Z[a + n * b];
      T[r + m * b] = s;
    }
  for (int s2 = 0; s2 < m; ++s2)
    for (int r = 0; r < m; ++r) {
      double s = 0;
      for (int b = 0; b < n; ++b) s += T[r + m * b] * R[s2 + ldr * b];
      out[r + m * s2] = s;
    }
}

/* out (n x n) (+)= L^T H (m x m) R, L, R: m x n */
static void contract_bwd(double *out, const double *L, int ldl, const double *R, int ldr, const double *H,
                         int m, int n, int accumulate) {
  double T[16 * 16];
  for (int s2 = 0; s2 < m; ++s2)
    for (int a = 0; a < n; ++a) {
      double s = 0;
      for (int r = 0; r < m; ++r) s += L[r + ldl * a] * H[r + m * s2];
      T[a + n * s2] = s;
    }
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) {
      double s = 0;
      for (int s2 = 0; s2 < m; ++s2) s += T[a + n * s2] * R[s2 + ldr * b];
      out[a + n * b] = accumulate ? out[a + n * b] + s : s;
    }
}

static double src_time(const or_pre *p, double t) {
  if (p->src_on && t < p->src_Ts) {
    double s = sin(M_PI * t / p->src_Ts);
    return sin(p->src_omega * t) * (s * s);
  }
  return 0.0;
}

/* _abc_face (rhs.jl:74-85) and _wall_face (rhs.jl:91-96) for one point */
static void side_flux(const or_pre *p, int s, double c2f, double af, double cf, double bf, double v_fp,
                      double gun, double gvn, double gu_ex, double gv_ex, double v_ex, double *F1,
                      double *dv) {
  if (p->kind[s] == 3) {
    double g2 = c2f * gu_ex + af * gv_ex;
    double rho_w = c2f * gun + af * gvn - g2;
    *dv = -(p->kap[s] / cf) * rho_w;
    *F1 = g2;
    return;
  }
  double g = p->gam[s], et = p->eta[s], sg = p->sig[s], kb = p->kb[s];
  double rho_num = et * (c2f * gun + af * gvn) + g * cf * sqrt(1.0 - kb * bf * v_fp) * v_fp;
  double rho_ex = et * (c2f * gu_ex + af * gv_ex) + g * cf * sqrt(1.0 - kb * bf * v_ex) * v_ex;
  double rho = rho_num - rho_ex;
  double sqf = sqrt(1.0 - kb * bf * v_fp);
  *F1 = c2f * gun + af * gvn - (et + sg * g) * rho;
  *dv = -(g - sg * et) / (cf * sqf) * rho;
}

/* One physical side, point by point (rhs.jl:738-765). Returns the smallest failure key or 0. */
static long boundary_side(or_ws *ws, int s, double ct, double st, double two_h) {
  const or_pre *p = &ws->p;
  int N = p->N, nq = p->nu;
  const double *c2a, *afa, *cfa, *bfa, *sp, *spn;
  double sgn;
  int slot, tix;
  int hz = s < 2;
  if (s == 0) { c2a = p->hc2; afa = p->haf; cfa = p->hcf; bfa = p->hbf; sp = p->bcB_sp; spn = p->bcB_spy; sgn = -1; slot = SB; }
  else if (s == 1) { c2a = p->hc2; afa = p->haf; cfa = p->hcf; bfa = p->hbf; sp = p->bcT_sp; spn = p->bcT_spy; sgn = 1; slot = ST; }
  else if (s == 2) { c2a = p->vc2; afa = p->vaf; cfa = p->vcf; bfa = p->vbf; sp = p->bcL_sp; spn = p->bcL_spx; sgn = -1; slot = SL; }
  else { c2a = p->vc2; afa = p->vaf; cfa = p->vcf; bfa = p->vbf; sp = p->bcR_sp; spn = p->bcR_spx; sgn = 1; slot = SR; }
  tix = slot;
  long key = 0;
  int wall = p->kind[s] == 3;
  for (int m = 0; m < N; ++m) {
    /* element and face indices of the side's m-th face */
    int j, k, fidx;
    if (s == 0) { j = 0; k = m; }
    else if (s == 1) { j = N - 1; k = m; }
    else if (s == 2) { j = m; k = 0; }
    else { j = m; k = N - 1; }
    size_t e = (size_t)j + (size_t)N * k;
    for (int i = 0; i < nq; ++i) {
      size_t I = i + (size_t)nq * e;
      if (hz) fidx = i + nq * ((s == 0 ? 0 : N) + (N + 1) * k);
      else fidx = i + nq * (j + N * (s == 2 ? 0 : N));
      double c2f = c2a[fidx], af = afa[fidx], cf = cfa[fidx], bf = bfa[fidx];
      double v_fp = ws->tr[T_V + tix][I];
      double gun = sgn * (two_h * ws->tr[T_DU + tix][I]);
      double gvn = sgn * (two_h * ws->tr[T_DV + tix][I]);
      double spn_i = spn[i + nq * m], sp_i = sp[i + nq * m];
      double gu_ex = sgn * (ct * spn_i - spn_i);
      double gv_ex = sgn * (-p->omega * st * spn_i);
      double v_ex = -p->omega * st * sp_i;
      if (!wall) {
        int check = (1.0 - p->kb[s] * bf * v_fp <= 0.0) ? 1 : (1.0 - p->kb[s] * bf * v_ex <= 0.0) ? 2 : 0;
        if (check) {
          long kk = 2L * ((long)s * nq * N + i + (long)m * nq) + check;
          key = key == 0 ? kk : (kk < key ? kk : key);
          continue;
        }
      }
      double F1, dv;
      side_flux(p, s, c2f, af, cf, bf, v_fp, gun, gvn, gu_ex, gv_ex, v_ex, &F1, &dv);
      ws->sl[S_A + slot][I] = F1;
      ws->sl[S_D + slot][I] = sgn * (af * dv);
      ws->sl[S_F + slot][I] = -sgn * (c2f * dv);
    }
  }
  return key;
}

/* interior faces (rhs.jl:620-700): horizontal (orient 0) or vertical (orient 1) */
static void interior_faces(or_ws *ws, int orient, double two_h) {
  const or_pre *p = &ws->p;
  int N = p->N, nq = p->nu;
  if (N < 2) return;
  double th = p->theta, tau = p->tau, lu = p->lu, lv = p->lv;
  int tm = orient ? SR : ST, tp = orient ? SL : SB; /* trace / slot side of "-" and "+" element */
  const double *c2p_a = orient ? p->vc2 : p->hc2, *afp_a = orient ? p->vaf : p->haf;
  const double *c2m_a = orient ? p->vc2m : p->hc2m, *afm_a = orient ? p->vafm : p->hafm;
  const double *jc_a = orient ? p->vJC : p->hJC;
#pragma omp parallel for schedule(static)
  for (int k = orient ? 1 : 0; k < N; ++k) {
    for (int j = orient ? 0 : 1; j < N; ++j) {
      int jm = orient ? j : j - 1, km = orient ? k - 1 : k;
      size_t ep = (size_t)j + (size_t)N * k, em = (size_t)jm + (size_t)N * km;
      for (int i = 0; i < nq; ++i) {
        size_t Ip = i + nq * ep, Im = i + nq * em;
        size_t f = orient ? i + (size_t)nq * (j + (size_t)N * k) : i + (size_t)nq * (j + (size_t)(N + 1) * k);
        double vm = ws->tr[T_V + tm][Im], vp = ws->tr[T_V + tp][Ip];
        double dum = ws->tr[T_DU + tm][Im], dup = ws->tr[T_DU + tp][Ip];
        double dvm = ws->tr[T_DV + tm][Im], dvp = ws->tr[T_DV + tp][Ip];
        double Ap, Dp, Fp, Am, Dm, Fm;
        if (p->one_sided) {
          double c2m = c2m_a[f], c2p = c2p_a[f], afm = afm_a[f], afp = afp_a[f], K = jc_a[f];
          double J = two_h * (c2m * dum - c2p * dup + afm * dvm - afp * dvp) + K;
          double G = two_h * ((1 - th) * (c2m * dum + afm * dvm) + th * (c2p * dup + afp * dvp));
          double pen = (0.5 * (c2m + c2p)) * lu + (0.5 * (afm + afp)) * lv;
          double s = vm - vp;
          double dvsp = th * s - tau * J, dvsm = (1 - th) * (vp - vm) - tau * J;
          Ap = pen * s - G - (1 - th) * K; Dp = -afp * dvsp; Fp = c2p * dvsp;
          Am = G - pen * s - th * K; Dm = afm * dvsm; Fm = -c2m * dvsm;
        } else {
          double c2 = c2p_a[f], af = afp_a[f];
          double gs = two_h * (c2 * (th * dup + (1 - th) * dum) + af * (th * dvp + (1 - th) * dvm));
          double Jt = c2 * (two_h * (dum - dup)) + af * (two_h * (dvm - dvp));
          double pen = c2 * lu + af * lv;
          Ap = pen * (vm - vp) - gs;
          Dp = -af * (th * (vm - vp) - tau * Jt);
          Fp = c2 * (th * (vm - vp) - tau * Jt);
          Am = gs - pen * (vm - vp);
          Dm = af * ((1 - th) * (vp - vm) - tau * Jt);
          Fm = -c2 * ((1 - th) * (vp - vm) - tau * Jt);
        }
        ws->sl[S_A + tp][Ip] = Ap; ws->sl[S_D + tp][Ip] = Dp; ws->sl[S_F + tp][Ip] = Fp;
        ws->sl[S_A + tm][Im] = Am; ws->sl[S_D + tm][Im] = Dm; ws->sl[S_F + tm][Im] = Fm;
      }
    }
  }
}

/* Chebyshev interval data on element e (rhs.jl:889-907); returns the step count, or -1 if not PD */
static int cheb_setup_elem(or_ws *ws, size_t e, const double *V) {
  const or_pre *p = &ws->p;
  int qh = p->qh, nv = p->nv;
  size_t E = (size_t)p->N * p->N;
  double *G = ws->G + (size_t)qh * qh * e;
  contract_fwd(G, p->P_h, qh, p->P_h, qh, V, qh, nv);
  double gmin = INFINITY, gmax = -INFINITY;
  int nan = 0;
  for (int s = 0; s < qh; ++s)
    for (int r = 0; r < qh; ++r) {
      double g = G[r + qh * s] * (2.0 * p->beta_hq[r + qh * (e + E * s)]);
      G[r + qh * s] = g;
      if (g != g) nan = 1;
      if (g < gmin) gmin = g;
      if (g > gmax) gmax = g;
    }
  double amin = 1.0 - gmax, amax = 1.0 - gmin;
  if (nan || !(amin > 0)) return -1;
  double th = 0.5 * (amax + amin);
  double de = fmax(0.5 * (amax - amin), 1e-15 * th);
  ws->th[e] = th; ws->de[e] = de; ws->s1[e] = th / de;
  for (int s = 0; s < qh; ++s)
    for (int r = 0; r < qh; ++r) G[r + qh * s] *= p->W_h[r + qh * s];
  double L = acosh(1.0 / p->mass_tol);
  return (int)ceil(L / acosh(ws->s1[e]));
}

/* Kd = P_h^T (G ∘ (P_h d P_h^T)) P_h */
static void apply_K(const or_pre *p, const double *G, const double *d, double *Kd) {
  int qh = p->qh, nv = p->nv;
  double Y[16 * 16];
  contract_fwd(Y, p->P_h, qh, p->P_h, qh, d, qh, nv);
  for (int i = 0; i < qh * qh; ++i) Y[i] *= G[i];
  contract_bwd(Kd, p->P_h, qh, p->P_h, qh, Y, qh, nv, 0);
}

/* CG on element e (rhs.jl:824-853): returns 0 ok, 1 not converged, -1 not PD */
static int cg_elem(const or_pre *p, size_t e, const double *V, const double *R, double *X) {
  int qh = p->qh, nv = p->nv, n2 = nv * nv;
  double G[16 * 16], r[256], pp[256], Ap[256];
  contract_fwd(G, p->P_h, qh, p->P_h, qh, V, qh, nv);
  const double *bh = p->beta_hE + (size_t)qh * qh * e;
  for (int i = 0; i < qh * qh; ++i) G[i] = 2.0 * bh[i] * G[i] * p->W_h[i];
  for (int i = 0; i < n2; ++i) X[i] = R[i];
  apply_K(p, G, X, r);
  for (int i = 0; i < n2; ++i) pp[i] = r[i];
  double rr = 0, r0 = 0;
  for (int i = 0; i < n2; ++i) { rr += r[i] * r[i]; r0 += R[i] * R[i]; }
  r0 = sqrt(r0);
  int it = 0, maxit = n2 + 10;
  while (sqrt(rr) > p->mass_tol * r0 && it < maxit) {
    ++it;
    apply_K(p, G, pp, Ap);
    for (int i = 0; i < n2; ++i) Ap[i] = pp[i] - Ap[i];
    double pAp = 0;
    for (int i = 0; i < n2; ++i) pAp += pp[i] * Ap[i];
    if (!(pAp > 0)) return -1;
    double a = rr / pAp;
    for (int i = 0; i < n2; ++i) { X[i] += a * pp[i]; r[i] -= a * Ap[i]; }
    double rrn = 0;
    for (int i = 0; i < n2; ++i) rrn += r[i] * r[i];
    for (int i = 0; i < n2; ++i) pp[i] = r[i] + (rrn / rr) * pp[i];
    rr = rrn;
  }
  return sqrt(rr) > p->mass_tol * r0 ? 1 : 0;
}

/*
 * One right-hand side evaluation (rhs.jl:498-550). Returns 0, 2 (boundary
 * weight; info[0] = key), 3 (mass matrix not PD; info[0] = 1-based element).
 * info[1] = Chebyshev steps, info[2] = CG systems above the tolerance.
 */
int or_rhs(or_ws *ws, const double *u, const double *v, double t, double *ut, double *vt, long *info) {
  const or_pre *p = &ws->p;
  int N = p->N, nu = p->nu, nv = p->nv, nq = p->nu, qh = p->qh;
  size_t E = (size_t)N * N;
  double h = 1.0 / N, two_h = 2.0 / h, four_hh = 4.0 / (h * h);
  double ct = p->mms_on ? cos(p->omega * t) : 0.0;
  double st = p->mms_on ? sin(p->omega * t) : 0.0;
  double srct = p->src_on ? src_time(p, t) : 0.0;
  info[0] = info[1] = info[2] = 0;
  long mfail = LONG_MAX;
  /* region 1: traces and Chebyshev intervals */
#pragma omp parallel for schedule(static) reduction(min : mfail)
  for (long e = 0; e < (long)E; ++e) {
    double U[256], V[256];
    load_elem(U, u, e, E, nu);
    load_elem(V, v, e, E, nv);
    size_t o = (size_t)nq * e;
    trace4(ws->tr[T_DU + SB] + o, ws->tr[T_DU + ST] + o, ws->tr[T_DU + SL] + o, ws->tr[T_DU + SR] + o,
           p->P_u, nq, nu, p->E1bl_u, p->E1br_u, U);
    trace4(ws->tr[T_V + SB] + o, ws->tr[T_V + ST] + o, ws->tr[T_V + SL] + o, ws->tr[T_V + SR] + o,
           p->P_u, nq, nv, p->Ebl_u, p->Ebr_u, V);
    trace4(ws->tr[T_DV + SB] + o, ws->tr[T_DV + ST] + o, ws->tr[T_DV + SL] + o, ws->tr[T_DV + SR] + o,
           p->P_u, nq, nv, p->E1bl_u, p->E1br_u, V);
    if (p->cheb) {
      int n = cheb_setup_elem(ws, e, V);
      ws->nst[e] = n;
      if (n < 0 && e + 1 < mfail) mfail = e + 1;
    }
  }
  /* region 2: faces and boundary */
  interior_faces(ws, 0, two_h);
  interior_faces(ws, 1, two_h);
  long key = 0;
  for (int s = 0; s < 4; ++s) {
    long k = boundary_side(ws, s, ct, st, two_h);
    if (k > 0) key = key == 0 ? k : (k < key ? k : key);
  }
  if (key > 0) { info[0] = key; return 2; }
  if (mfail != LONG_MAX) { info[0] = mfail; return 3; }
  int nsteps = 1;
  if (p->cheb)
    for (size_t e = 0; e < E; ++e)
      if (ws->nst[e] > nsteps) nsteps = ws->nst[e];
  info[1] = nsteps;
  /* region 3: volume, source, lifts, u-equation, mass solve */
  long cgfail = 0, cgbad = LONG_MAX;
#pragma omp parallel for schedule(static) reduction(+ : cgfail) reduction(min : cgbad)
  for (long e = 0; e < (long)E; ++e) {
    double U[256], V[256], G1[256], G2[256], H1[256], H2[256];
    const double *P_u = p->P_u, *S_u = p->S_u;
    load_elem(U, u, e, E, nu);
    load_elem(V, v, e, E, nv);
    double *R = ws->Rv + (size_t)nv * nv * e, *B = ws->VB + (size_t)nu * nu * e;
    /* volume terms (rhs.jl:317-333) */
    contract_fwd(G1, S_u, nq, P_u, nq, U, nq, nu);
    contract_fwd(G2, P_u, nq, S_u, nq, U, nq, nu);
    for (int s = 0; s < nq; ++s)
      for (int r = 0; r < nq; ++r) {
        double c = p->Cw[r + nq * (e + E * s)];
        H1[r + nq * s] = c * G1[r + nq * s];
        H2[r + nq * s] = c * G2[r + nq * s];
      }
    contract_fwd(G1, S_u, nq, P_u, nq, V, nq, nv);
    contract_fwd(G2, P_u, nq, S_u, nq, V, nq, nv);
    for (int s = 0; s < nq; ++s)
      for (int r = 0; r < nq; ++r) {
        double a = p->Aw[r + nq * (e + E * s)];
        H1[r + nq * s] += a * G1[r + nq * s];
        H2[r + nq * s] += a * G2[r + nq * s];
      }
    contract_bwd(R, S_u, nq, P_u, nq, H1, nq, nv, 0);
    contract_bwd(R, P_u, nq, S_u, nq, H2, nq, nv, 1);
    for (int s = 0; s < nq; ++s)
      for (int r = 0; r < nq; ++r) {
        double c = p->Cw[r + nq * (e + E * s)];
        G1[r + nq * s] *= c;
        G2[r + nq * s] *= c;
      }
    contract_bwd(B, S_u, nq, P_u, nq, G1, nq, nu, 0);
    contract_bwd(B, P_u, nq, S_u, nq, G2, nq, nu, 1);
    /* source (rhs.jl:340-350) */
    double om = p->omega;
    for (int i = 0; i < nv * nv; ++i) {
      size_t l = i + (size_t)nv * nv * e;
      double rv = (-four_hh) * R[i] + (-om * om * ct) * p->PiSP[l] + (-2.0 * om * om * om * st * ct) * p->PiBSP2[l] +
                  (1.0 - ct) * p->PiCdiv[l] + (om * st) * p->PiDdiv[l];
      if (p->src_on) rv += srct * p->src_projE[l];
      R[i] = rv;
    }
    /* lifts (rhs.jl:421-473) */
    double *F = ws->Fu + (size_t)nu * nu * e;
    for (int i = 0; i < nu * nu; ++i) F[i] = 0.0;
    for (int side = 0; side < 4; ++side) {
      const double *A = ws->sl[S_A + side] + (size_t)nq * e, *D = ws->sl[S_D + side] + (size_t)nq * e,
                   *Fs = ws->sl[S_F + side] + (size_t)nq * e;
      const double *Ev = (side == SB || side == SL) ? p->Ebl_u : p->Ebr_u;
      const double *E1 = (side == SB || side == SL) ? p->E1bl_u : p->E1br_u;
      int hz = side < 2;
      double YA[16], YD[16], YF[16];
      for (int b = 0; b < nv; ++b) {
        double sA = 0, sD = 0;
        for (int i = 0; i < nq; ++i) {
          sA += P_u[i + nq * b] * (p->w[i] * A[i]);
          sD += P_u[i + nq * b] * (p->w[i] * D[i]);
        }
        YA[b] = sA; YD[b] = sD;
      }
      for (int b = 0; b < nu; ++b) {
        double sF = 0;
        for (int i = 0; i < nq; ++i) sF += P_u[i + nq * b] * (p->w[i] * Fs[i]);
        YF[b] = sF;
      }
      for (int b = 0; b < nv; ++b)
        for (int a = 0; a < nv; ++a) {
          int kk = a + nv * b;
          if (hz) { R[kk] = R[kk] + (two_h * Ev[a]) * YA[b]; R[kk] = R[kk] + (four_hh * E1[a]) * YD[b]; }
          else { R[kk] = R[kk] + (two_h * YA[a]) * Ev[b]; R[kk] = R[kk] + (four_hh * YD[a]) * E1[b]; }
        }
      for (int b = 0; b < nu; ++b)
        for (int a = 0; a < nu; ++a) {
          int kk = a + nu * b;
          F[kk] = F[kk] + (hz ? E1[a] * YF[b] : YF[a] * E1[b]);
        }
    }
    /* u-equation with the packed symmetric inverse (rhs.jl:361-382) */
    {
      int n = nu * nu;
      size_t ntri = (size_t)n * (n + 1) / 2;
      const double *Ai = p->Ainv + ntri * e;
      double b[256], *X = ws->UT + (size_t)n * e;
      for (int i = 0; i < n; ++i) { b[i] = B[i] - F[i]; X[i] = 0.0; }
      b[0] += V[0];
      for (int j = 0; j < n; ++j) {
        double bj = b[j], s = 0.0;
        size_t off = (size_t)j * (j + 1) / 2;
        for (int i = 0; i < j; ++i) {
          double a = Ai[off + i];
          X[i] += a * bj;
          s += a * b[i];
        }
        X[j] = Ai[off + j] * bj + (X[j] + s);
      }
    }
    /* mass system */
    double *X = ws->VT + (size_t)nv * nv * e;
    if (p->cheb) {
      /* n Chebyshev steps (rhs.jl:921-939) */
      int n2 = nv * nv;
      double r[256], d[256], Kd[256];
      const double *Ge = ws->G + (size_t)qh * qh * e;
      double th = ws->th[e], de = ws->de[e], s1 = ws->s1[e];
      double rho = 1.0 / s1;
      for (int i = 0; i < n2; ++i) { r[i] = R[i]; d[i] = r[i] / th; X[i] = 0.0; }
      for (int step = 1; step <= nsteps; ++step) {
        for (int i = 0; i < n2; ++i) X[i] += d[i];
        if (step == nsteps) break;
        apply_K(p, Ge, d, Kd);
        for (int i = 0; i < n2; ++i) r[i] -= d[i] - Kd[i];
        double rhon = 1.0 / (2.0 * s1 - rho);
        for (int i = 0; i < n2; ++i) d[i] = (rhon * rho) * d[i] + (2.0 * rhon / de) * r[i];
        rho = rhon;
      }
    } else {
      int rc = cg_elem(p, e, V, R, X);
      if (rc > 0) cgfail += 1;
      if (rc < 0 && e + 1 < cgbad) cgbad = e + 1;
    }
  }
  if (cgbad != LONG_MAX) { info[0] = cgbad; return 3; }
  info[2] = cgfail;
  /* to the state layout (rhs.jl:282-288) */
#pragma omp parallel for schedule(static)
  for (long e = 0; e < (long)E; ++e) {
    for (int b = 0; b < nu; ++b)
      for (int a = 0; a < nu; ++a) ut[e + E * (a + (size_t)nu * b)] = ws->UT[a + nu * b + (size_t)nu * nu * e];
    for (int b = 0; b < nv; ++b)
      for (int a = 0; a < nv; ++a) vt[e + E * (a + (size_t)nv * b)] = ws->VT[a + nv * b + (size_t)nv * nv * e];
  }
  return 0;
}

/* rk4_step! (solver.jl:289-321). info as or_rhs; info[3] = all entries finite. */
int or_rk4_step(or_ws *ws, double *u, double *v, double t, double dt, long *info) {
  const or_pre *p = &ws->p;
  size_t E = (size_t)p->N * p->N, nU = E * p->nu * p->nu, nV = E * p->nv * p->nv;
  double cs[3] = {0.5 * dt, 0.5 * dt, dt}, ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
  long maxn = 0, cgf = 0;
  for (int s = 0; s < 4; ++s) {
    const double *xu = s == 0 ? u : ws->su, *xv = s == 0 ? v : ws->sv;
    int rc = or_rhs(ws, xu, xv, ts[s], ws->k[s][0], ws->k[s][1], info);
    if (rc) return rc;
    if (info[1] > maxn) maxn = info[1];
    cgf += info[2];
    if (s < 3) {
      double c = cs[s];
#pragma omp parallel for schedule(static)
      for (long i = 0; i < (long)nU; ++i) ws->su[i] = u[i] + c * ws->k[s][0][i];
#pragma omp parallel for schedule(static)
      for (long i = 0; i < (long)nV; ++i) ws->sv[i] = v[i] + c * ws->k[s][1][i];
    }
  }
  double c = dt / 6.0;
  int fin = 1;
#pragma omp parallel for schedule(static) reduction(&& : fin)
  for (long i = 0; i < (long)nU; ++i) {
    u[i] = u[i] + c * (((ws->k[0][0][i] + 2.0 * ws->k[1][0][i]) + 2.0 * ws->k[2][0][i]) + ws->k[3][0][i]);
    fin = fin && isfinite(u[i]);
  }
#pragma omp parallel for schedule(static) reduction(&& : fin)
  for (long i = 0; i < (long)nV; ++i) {
    v[i] = v[i] + c * (((ws->k[0][1][i] + 2.0 * ws->k[1][1][i]) + 2.0 * ws->k[2][1][i]) + ws->k[3][1][i]);
    fin = fin && isfinite(v[i]);
  }
  info[1] = maxn;
  info[2] = cgf;
  info[3] = fin;
  return 0;
}

/* Several steps from t0 (dt fixed); stops at the first error. Returns the code; info[4] = steps done. */
int or_rk4_steps(or_ws *ws, double *u, double *v, double t0, double dt, long nsteps, long *info) {
  double t = t0;
  info[4] = 0;
  for (long it = 0; it < nsteps; ++it) {
    int rc = or_rk4_step(ws, u, v, t, dt, info);
    if (rc) return rc;
    t += dt;
    info[4] = it + 1;
  }
  return 0;
}

int or_max_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
