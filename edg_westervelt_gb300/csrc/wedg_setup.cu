// Set-up kernels of wedg_create and wedg_create_points: the packed inverses of the pinned
// c²-stiffness of every element (src/solver.jl:528-535), computed on the device from the
// element's c²W at the u-quadrature points when the caller passes no Ainv_u; and the arrays of
// `pre` (element matrices, one-sided face arrays, jump terms, projections) built from the point
// values of the coefficients and data (src/solver.jl:509-552, 554-602, 647-662, 698-770).
//
// One block per element, the n × n matrix (n = (q_u+1)² ≤ 64) in shared memory:
//   M = Φξᵀ diag(c²W) Φξ + Φηᵀ diag(c²W) Φη, M[0][0] += 1, with Φξ = P_u ⊗ S_u, Φη = S_u ⊗ P_u
//   (Kronecker products in numpy's `kron` index order: row p1 nq + p2, column i1 nu + i2);
//   M = L Lᵀ (Cholesky, right-looking); Li = L⁻¹ (forward substitution, a column per thread);
//   A = Liᵀ Li, written as the packed upper triangle by columns, row j(j+1)/2 + i, [row E + e].
// A pivot that is not positive sets the element's flag (the reference's cholesky throws).
#include <cuda_runtime.h>

#include "wedg_setup.h"

namespace wedg {

__global__ void k_ainv(const double *Cw, int E, int nu, const double *Pu, const double *Su, double *Ainv,
                       unsigned int *bad) {
  extern __shared__ double sh[];
  const int e = blockIdx.x;
  if (e >= E) return;
  const int nq = nu, n = nu * nu, np = nq * nq;
  double *M = sh, *Li = sh + n * n, *cw = Li + n * n, *P = cw + np, *S = P + nq * nu;
  __shared__ int fail;
  const int t = threadIdx.x, T = blockDim.x;
  if (t == 0) fail = 0;
  for (int i = t; i < np; i += T) cw[i] = Cw[(size_t)i * E + e];
  for (int i = t; i < nq * nu; i += T) { P[i] = Pu[i]; S[i] = Su[i]; }   // [p + nq d], column-major
  __syncthreads();
  // ---- assembly (upper triangle computed, mirrored)
  for (int idx = t; idx < n * n; idx += T) {
    const int i = idx % n, j = idx / n;
    if (i > j) continue;
    const int i1 = i / nu, i2 = i % nu, j1 = j / nu, j2 = j % nu;
    double s = 0.0;
    for (int p1 = 0; p1 < nq; ++p1) {
      const double pa = P[p1 + nq * i1] * P[p1 + nq * j1], sa = S[p1 + nq * i1] * S[p1 + nq * j1];
      for (int p2 = 0; p2 < nq; ++p2) {
        const double c = cw[p1 * nq + p2];
        s = fma(c, pa * (S[p2 + nq * i2] * S[p2 + nq * j2]) + sa * (P[p2 + nq * i2] * P[p2 + nq * j2]), s);
      }
    }
    if (i == 0 && j == 0) s += 1.0;
    M[i + n * j] = s;
    M[j + n * i] = s;
  }
  __syncthreads();
  // ---- Cholesky: L in the lower triangle of M
  for (int k = 0; k < n; ++k) {
    if (t == 0) {
      const double d = M[k + n * k];
      if (!(d > 0.0)) fail = 1;
      M[k + n * k] = sqrt(d > 0.0 ? d : 1.0);
    }
    __syncthreads();
    const double lkk = M[k + n * k];
    for (int i = k + 1 + t; i < n; i += T) M[i + n * k] /= lkk;
    __syncthreads();
    const int m = n - k - 1;
    for (int idx = t; idx < m * m; idx += T) {
      const int i = k + 1 + idx % m, j = k + 1 + idx / m;
      if (j <= i) M[i + n * j] = fma(-M[i + n * k], M[j + n * k], M[i + n * j]);
    }
    __syncthreads();
  }
  // ---- Li = L⁻¹ (lower triangular), one column c per thread
  for (int c = t; c < n; c += T) {
    for (int i = 0; i < c; ++i) Li[i + n * c] = 0.0;
    for (int i = c; i < n; ++i) {
      double s = (i == c) ? 1.0 : 0.0;
      for (int k = c; k < i; ++k) s = fma(-M[i + n * k], Li[k + n * c], s);
      Li[i + n * c] = s / M[i + n * i];
    }
  }
  __syncthreads();
  // ---- A = Liᵀ Li, packed upper triangle by columns
  for (int idx = t; idx < n * n; idx += T) {
    const int i = idx % n, j = idx / n;
    if (i > j) continue;
    double s = 0.0;
    for (int k = j; k < n; ++k) s = fma(Li[k + n * i], Li[k + n * j], s);
    Ainv[(size_t)(j * (j + 1) / 2 + i) * E + e] = s;
  }
  if (t == 0 && fail) atomicAdd(bad, 1u);
}

size_t ainv_smem(int nu) {
  const int n = nu * nu, nq = nu;
  return sizeof(double) * (2 * (size_t)n * n + nq * nq + 2 * nq * nu);
}

// ---------------------------------------------------------------------------------------------
// The rest of `pre` on the device (wedg_create_points): the arithmetic is the host's (the same
// products in the same order; __dmul_rn / __dadd_rn where the host rounds a product before a sum,
// so that no contraction into an FMA changes a comparison)
// ---------------------------------------------------------------------------------------------

// the coordinates of u-point (r, s) of element e = j + N k
#define PTS_XY(r, s) const double x = g.xq[k + (size_t)g.N * (s)], y = g.yq[j + (size_t)g.N * (r)]

__global__ void k_pts_check(PtsField c_q, PtsField a_q, PtsGrid g, const double *w, int nq, int E, unsigned *flags) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int j = e % g.N, k = e / g.N;
  const size_t Eu = (size_t)E;
  const double w00 = __dmul_rn(w[0], w[0]);
  double c0, a0;
  {
    PTS_XY(0, 0);
    c0 = c_q.at(e, x, y);
    a0 = a_q.at(e, x, y);
  }
  const double c2 = __dmul_rn(__dmul_rn(c0, c0), w00) / w00, al = __dmul_rn(a0, w00) / w00;
  bool ok = c2 > 0.0;
  for (int s = 0; s < nq && ok; ++s)
    for (int r = 0; r < nq; ++r) {
      const double W = __dmul_rn(w[r], w[s]);
      PTS_XY(r, s);
      const double c = c_q.at(e + Eu * (r + nq * s), x, y), a = a_q.at(e + Eu * (r + nq * s), x, y);
      const double cw = __dmul_rn(__dmul_rn(c, c), W), aw = __dmul_rn(a, W);
      if (fabs(cw - __dmul_rn(c2, W)) > __dmul_rn(1e-14, fabs(cw)) ||
          fabs(aw - __dmul_rn(al, W)) > __dmul_rn(1e-14, fabs(aw))) {
        ok = false;
        break;
      }
    }
  if (!ok) atomicOr(flags, (unsigned)PTS_NOT_CONSTANT);
}

__global__ void k_pts_elem(PtsField c_q, PtsField a_q, PtsGrid g, const double *w, int nq, int E, double *c2e,
                           double *ae, double *ic2e, double *Cw, double *Aw) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int j = e % g.N, k = e / g.N;
  const size_t Eu = (size_t)E;
  if (c2e) {
    const double w00 = __dmul_rn(w[0], w[0]);
    PTS_XY(0, 0);
    const double c0 = c_q.at(e, x, y), a0 = a_q.at(e, x, y);
    const double c2 = __dmul_rn(__dmul_rn(c0, c0), w00) / w00;
    c2e[e] = c2;
    ae[e] = __dmul_rn(a0, w00) / w00;
    ic2e[e] = 1.0 / c2;
  }
  if (Cw)
    for (int s = 0; s < nq; ++s)
      for (int r = 0; r < nq; ++r) {
        const size_t l = e + Eu * (r + nq * s);
        const double W = __dmul_rn(w[r], w[s]);
        PTS_XY(r, s);
        const double c = c_q.at(l, x, y);
        Cw[l] = __dmul_rn(__dmul_rn(c, c), W);
        Aw[l] = __dmul_rn(a_q.at(l, x, y), W);
      }
}

// The value of a family seen from below (lower = true: the "-" side) or above a face point
// (src/solver.jl:389-392): the plain value where the family is continuous there to the tolerance
// A family's value at a point (x, y) when it is a table
__device__ __forceinline__ double pts_cell(const PtsFace &f, double x, double y) {
  int r = (int)floor((double)f.m * y), c = (int)floor((double)f.n * x);
  r = r < 0 ? 0 : r > f.m - 1 ? f.m - 1 : r;
  c = c < 0 ? 0 : c > f.n - 1 ? f.n - 1 : c;
  return f.tab[r * f.n + c];
}

// The three values of a family at face point pin (array families) or at its coordinates: (x, y)
// the point, (xl, yl) and (xh, yh) the points δ below / above it (the point itself outside the domain)
struct PtsTriple {
  double h0, hm, hp;
};
__device__ __forceinline__ PtsTriple pts_triple(const PtsFace &f, size_t pin, double x, double y, double xl,
                                                double yl, double xu, double yu) {
  if (f.at) return PtsTriple{f.at[pin], f.lo[pin], f.hi[pin]};
  if (f.tab) return PtsTriple{pts_cell(f, x, y), pts_cell(f, xl, yl), pts_cell(f, xu, yu)};
  return PtsTriple{f.value, f.value, f.value};
}

__device__ __forceinline__ double pts_side(const PtsFace &f, const PtsTriple &v, bool lower) {
  if (!f.at && !f.tab) return f.value;
  const double h0 = v.h0, hm = v.hm, hp = v.hp;
  const bool nm = fabs(hm - h0) <= __dadd_rn(__dmul_rn(1e-8, fmax(fabs(hm), fabs(h0))), f.s);
  const bool np = fabs(hp - h0) <= __dadd_rn(__dmul_rn(1e-8, fmax(fabs(hp), fabs(h0))), f.s);
  const bool use0 = isfinite(h0) && nm && np;
  return use0 ? h0 : (lower ? hm : hp);
}

__global__ void k_pts_faces(int N, int nq, bool hor, PtsGrid g, PtsFace c, PtsFace a, PtsFace b, PtsFace g0,
                            PtsFaceOut o, unsigned *flags) {
  const size_t nf = (size_t)nq * (N + 1) * N;
  unsigned fl = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nf; t += (size_t)gridDim.x * blockDim.x) {
    // t walks the output layout: h-faces [jf + (N+1)(k + N i)], v-faces [j + N (kf + (N+1) i)]
    int f, m, i;                  // f: the face index across (jf or kf), m: the element along it, i: point
    if (hor) {
      f = (int)(t % (N + 1));
      m = (int)((t / (N + 1)) % N);
      i = (int)(t / ((size_t)(N + 1) * N));
    } else {
      m = (int)(t % N);
      f = (int)((t / N) % (N + 1));
      i = (int)(t / ((size_t)N * (N + 1)));
    }
    const size_t pin = hor ? i + (size_t)nq * (f + (size_t)(N + 1) * m) : i + (size_t)nq * (m + (size_t)N * f);
    // the point and δ across the face (src/solver.jl:381-386): y = jf h ± δ on horizontal faces,
    // x = kf h ± δ on vertical ones; the face's own value outside the domain
    const double d = 0x1p-40, fh = (double)f * g.h;
    const double along = g.xq ? (hor ? g.xq[m + (size_t)N * i] : g.yq[m + (size_t)N * i]) : 0.0;
    const double x = hor ? along : fh, y = hor ? fh : along;
    const double lo = f > 0 ? fh - d : fh, up = f < N ? fh + d : fh;
    const double xl = hor ? x : lo, yl = hor ? lo : y, xu = hor ? x : up, yu = hor ? up : y;
    // the "+" array takes the value above face f (inside element f), the last face the one below
    // it; the "-" array the value below face f, the first face the one above it
    const bool plus_lower = f == N, minus_lower = f != 0;
    const PtsTriple vc = pts_triple(c, pin, x, y, xl, yl, xu, yu), va = pts_triple(a, pin, x, y, xl, yl, xu, yu);
    const double cp = pts_side(c, vc, plus_lower), cm = pts_side(c, vc, minus_lower);
    const double ap = pts_side(a, va, plus_lower), am = pts_side(a, va, minus_lower);
    const double c2p = __dmul_rn(cp, cp), c2m = __dmul_rn(cm, cm);
    o.c2[t] = c2p;
    o.c2m[t] = c2m;
    o.cf[t] = cp;
    o.af[t] = ap;
    o.afm[t] = am;
    o.bf[t] = pts_side(b, pts_triple(b, pin, x, y, xl, yl, xu, yu), plus_lower);
    double jc = 0.0;
    if ((g0.at || g0.value != 0.0) && f != 0 && f != N) {
      const PtsTriple vg = pts_triple(g0, pin, x, y, xl, yl, xu, yu);
      const double gp = pts_side(g0, vg, plus_lower), gm = pts_side(g0, vg, minus_lower);
      jc = __dmul_rn(c2m, gm) - __dmul_rn(c2p, gp);
    }
    o.JC[t] = jc;
    if (c2m != c2p || am != ap) fl |= PTS_JUMPS;
    if (jc != 0.0) fl |= PTS_JC;
  }
  if (fl) atomicOr(flags, fl);
}

__global__ void k_pts_face_max(int N, int nq, PtsGrid g, PtsFace fam, unsigned long long *out) {
  const size_t nf = (size_t)nq * (N + 1) * N;
  double best = 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < 2 * nf; t += (size_t)gridDim.x * blockDim.x) {
    const bool hor = t < nf;
    const size_t u = hor ? t : t - nf;
    const int f = (int)(u % (N + 1)), m = (int)((u / (N + 1)) % N), i = (int)(u / ((size_t)(N + 1) * N));
    const double d = 0x1p-40, fh = (double)f * g.h;
    const double along = hor ? g.xq[m + (size_t)N * i] : g.yq[m + (size_t)N * i];
    double v[2];
    int nv = 0;
    if (f > 0) v[nv++] = hor ? pts_cell(fam, along, fh - d) : pts_cell(fam, fh - d, along);
    if (f < N) v[nv++] = hor ? pts_cell(fam, along, fh + d) : pts_cell(fam, fh + d, along);
    for (int x = 0; x < nv; ++x)
      if (isfinite(v[x])) best = fmax(best, fabs(v[x]));
  }
  atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

__global__ void k_pts_proj(PtsGrid g, int qh, int nv, const double *Ph, const double *Wh, PtsProj p, double *out) {
  const int N = g.N, E = N * N;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int j = e % N, k = e / N;
  const size_t Eu = (size_t)E;
  double T[12][8];                 // T[r][b] = Σ_s W[r, s] X[r, s] P_h[s, b]  (qh ≤ 12, nv ≤ 8)
  for (int r = 0; r < qh; ++r) {
    for (int bb = 0; bb < nv; ++bb) T[r][bb] = 0.0;
    for (int s = 0; s < qh; ++s) {
      double x;
      const double xp = g.xh ? g.xh[k + (size_t)N * s] : 0.0, yp = g.yh ? g.yh[j + (size_t)N * r] : 0.0;
      if (p.kind == 2) {
        const double dx = xp - p.x0, dy = yp - p.y0;
        x = __dmul_rn(p.amp, exp(-__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) / __dmul_rn(p.r0, p.r0)));
      } else {
        x = p.x1[e + Eu * (r + qh * s)];
        if (p.kind == 1) x = __dmul_rn(p.x2.at(e + Eu * (r + qh * s), xp, yp), __dmul_rn(x, x));
      }
      const double wx = __dmul_rn(Wh[r + qh * s], x);
      for (int bb = 0; bb < nv; ++bb) T[r][bb] = fma(wx, Ph[s + qh * bb], T[r][bb]);
    }
  }
  for (int bb = 0; bb < nv; ++bb)
    for (int a = 0; a < nv; ++a) {
      double z = 0.0;
      for (int r = 0; r < qh; ++r) z = fma(Ph[r + qh * a], T[r][bb], z);
      out[(a + (size_t)nv * bb) * Eu + e] = z;
    }
}

__global__ void k_pts_beta2(PtsGrid g, int qh, PtsField b, double *out) {
  const size_t E = (size_t)g.N * g.N, n = E * qh * qh;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t e = i % E, rs = i / E, r = rs % qh, s = rs / qh, j = e % g.N, k = e / g.N;
    const double x = g.xh[k + g.N * s], y = g.yh[j + g.N * r];
    out[i] = 2.0 * b.at(i, x, y);
  }
}

}  // namespace wedg
