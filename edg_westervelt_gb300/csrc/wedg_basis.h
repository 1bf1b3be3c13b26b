// The 1D operators the kernels take as launch parameters, built on the host from
// the reference's `pre` (src/solver.jl:428-520): the u-quadrature (w, P_u, S_u),
// the face values of the basis (Ebl_u ... E1br_u), the high-order v-quadrature
// (P_h_v, W2d_h), and, for the constant-coefficient kernels, the 1D stiffness
// K1 = S^T diag(w) S with its eigenbasis; some of them with the quadrature
// weights or the mesh factors 2/h, 4/h² folded in.
//
// Both quadratures are Gauss-Legendre rules and the basis is the Legendre one
// (src/solver.jl:436-486), so every operator has a mirror parity: at the point
// mirrored through the element centre, mode d of the basis changes sign by
// (-1)^d and its derivative by (-1)^(d+1). The kernels use this to contract
// over half of the points (the even and odd modes of a point pair are a sum and
// a difference), and K1 couples only modes of equal parity. build_basis checks
// the parities of the given arrays to 1e-13 of their largest entry, then makes
// them exact (the second half of each rule is the mirror of the first, K1 and
// its eigenvectors are zero between modes of unlike parity); a rule that is not
// mirror-symmetric is refused. The changes are of the order of the arrays'
// own round-off (the reference builds the nodes by an eigen-decomposition that
// mirrors them to about 1e-16).
#pragma once
#include <cmath>

#include "../../include/wedg.h"
#include "wedg_dispatch.h"

namespace wedg {

// Cyclic Jacobi eigen-decomposition of the symmetric m×m block A (m < MAXN):
// A = Q diag(lam) Q^T. Entries of A that are exactly zero stay zero in every
// rotation that does not involve their row or column, so a block-diagonal A
// (after a permutation) gives a block-diagonal Q.
inline void jacobi_eig(int m, double A[MAXN][MAXN], double Q[MAXN][MAXN], double lam[MAXN]) {
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) Q[i][j] = i == j;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) off += A[p][q] * A[p][q];
    if (off < 1e-40) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        if (std::fabs(A[p][q]) < 1e-300) continue;
        const double tau = (A[q][q] - A[p][p]) / (2 * A[p][q]);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
        const double c = 1 / std::sqrt(1 + t * t), s = t * c;
        for (int k = 0; k < m; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {
          const double qkp = Q[k][p], qkq = Q[k][q];
          Q[k][p] = c * qkp - s * qkq;
          Q[k][q] = s * qkp + c * qkq;
        }
      }
  }
  for (int i = 0; i < m; ++i) lam[i] = A[i][i];
}

// Checks x[n-1-i] = sg x[i] to `tol` and makes it exact (x[n-1-i] := sg x[i] for i < n/2,
// the middle entry of an odd rule := 0 when sg = -1). x is read with stride `st`.
inline bool mirror(double *x, int n, int st, double sg, double tol) {
  for (int i = 0; i < (n + 1) / 2; ++i) {
    const double a = x[i * st], b = x[(n - 1 - i) * st];
    if (!(std::fabs(b - sg * a) <= tol)) return false;
  }
  for (int i = 0; i < n / 2; ++i) x[(n - 1 - i) * st] = sg * x[i * st];
  if ((n & 1) && sg < 0) x[(n / 2) * st] = 0.0;
  return true;
}

// Fills `bh` from `pre`; returns nullptr, or why the arrays are refused.
inline const char *build_basis(const wedg_config *cfg, const wedg_pre *pre, BasisHost &bh) {
  const int nu = cfg->qu1, nv = cfg->qv1, nq = nu, qh = cfg->q_high;
  bh = BasisHost{};
  bh.nu = nu; bh.nv = nv; bh.qh = qh;
  for (int i = 0; i < nq; ++i) {
    bh.w[i] = pre->w[i];
    for (int d = 0; d < nu; ++d) { bh.P[i][d] = pre->P_u[i + nq * d]; bh.S[i][d] = pre->S_u[i + nq * d]; }
  }
  for (int d = 0; d < nu; ++d) {
    bh.El[d] = pre->Ebl_u[d]; bh.Er[d] = pre->Ebr_u[d]; bh.E1l[d] = pre->E1bl_u[d]; bh.E1r[d] = pre->E1br_u[d];
  }
  for (int r = 0; r < qh; ++r) {
    for (int d = 0; d < nv; ++d) bh.Ph[r][d] = pre->P_h_v[r + qh * d];
    for (int s = 0; s < qh; ++s) bh.Wh[r][s] = pre->W2d_h[r + qh * s];
  }

  // ---- mirror parities, to 1e-13 of the largest entry of each array
  auto scale = [](const double *x, int n) {
    double m = 0;
    for (int i = 0; i < n; ++i) m = std::fmax(m, std::fabs(x[i]));
    return 1e-13 * m;
  };
  const char *asym = "the quadrature rules are not mirror-symmetric (Gauss-Legendre points and a Legendre basis "
                     "are required)";
  if (!mirror(bh.w, nq, 1, 1.0, scale(bh.w, nq))) return asym;
  const double tP = scale(&bh.P[0][0], MAXN * MAXN), tS = scale(&bh.S[0][0], MAXN * MAXN);
  const double tPh = scale(&bh.Ph[0][0], MAXQH * MAXN), tWh = scale(&bh.Wh[0][0], MAXQH * MAXQH);
  for (int d = 0; d < nu; ++d) {
    const double sg = (d & 1) ? -1.0 : 1.0;
    if (!mirror(&bh.P[0][d], nq, MAXN, sg, tP) || !mirror(&bh.S[0][d], nq, MAXN, -sg, tS)) return asym;
    // values and derivatives of mode d at the right end are ±those at the left end
    const double tE = 1e-13 * std::fmax(std::fabs(bh.El[d]), std::fabs(bh.Er[d]));
    const double tE1 = 1e-13 * std::fmax(std::fabs(bh.E1l[d]), std::fabs(bh.E1r[d]));
    if (!(std::fabs(bh.Er[d] - sg * bh.El[d]) <= tE) || !(std::fabs(bh.E1r[d] + sg * bh.E1l[d]) <= tE1))
      return asym;
    bh.Er[d] = sg * bh.El[d];
    bh.E1r[d] = -sg * bh.E1l[d];
  }
  for (int d = 0; d < nv; ++d)
    if (!mirror(&bh.Ph[0][d], qh, MAXN, (d & 1) ? -1.0 : 1.0, tPh)) return asym;
  for (int s = 0; s < qh; ++s)                       // W2d_h = w_h w_h^T: mirrored in both indices
    if (!mirror(&bh.Wh[0][s], qh, MAXQH, 1.0, tWh)) return asym;
  for (int r = 0; r < qh; ++r)
    if (!mirror(&bh.Wh[r][0], qh, 1, 1.0, tWh)) return asym;

  // ---- weights folded into the bases: W2d_h = w_h w_h^T (the kernels weight the point values
  //      by w_h[s] on the way back to the modes), w P_u, and the lift factor -E1l of the u-slots.
  //      Nothing here depends on the mesh size (the kernels take 2/h and 4/h² from the
  //      workspace), so instances of any N with the same degrees share these operators.
  for (int r = 0; r < qh; ++r) bh.wh[r] = std::sqrt(bh.Wh[r][r]);
  for (int r = 0; r < qh; ++r)
    for (int s = 0; s < qh; ++s)
      if (!(std::fabs(bh.wh[r] * bh.wh[s] - bh.Wh[r][s]) <= 1e-14 * std::fabs(bh.Wh[r][s])))
        return "W2d_h is not the outer product of one-dimensional weights";
  for (int r = 0; r < qh; ++r)
    for (int d = 0; d < nv; ++d) bh.PhW[r][d] = bh.wh[r] * bh.Ph[r][d];
  for (int i = 0; i < nq; ++i)
    for (int d = 0; d < nu; ++d) bh.Pw[i][d] = bh.w[i] * bh.P[i][d];
  for (int d = 0; d < nu; ++d) bh.E1F[d] = -bh.E1l[d];

  // ---- K1 = S^T diag(w) S: zero between modes of unlike parity, and in the first row and
  //      column (the constant mode has no derivative)
  for (int a = 0; a < nu; ++a)
    for (int c = 0; c < nu; ++c) {
      double s = 0;
      for (int i = 0; i < nq; ++i) s += bh.S[i][a] * bh.w[i] * bh.S[i][c];
      bh.K1[a][c] = ((a + c) & 1) || a == 0 || c == 0 ? 0.0 : s;
    }
  for (int a = 1; a < nu; ++a)
    for (int c = a + 1; c < nu; ++c) bh.K1[a][c] = bh.K1[c][a] = 0.5 * (bh.K1[a][c] + bh.K1[c][a]);

  // ---- eigenbasis of the nonsingular block K1[1:, 1:]; Q = diag(1, Q'). Every eigenvector lives
  //      on the modes of one parity; it is stored in a column of that parity (the odd and the even
  //      modes 1..nu-1 are as many as the eigenvectors on them), so that Q[a][c] = 0 for a + c odd.
  {
    const int m = nu - 1;
    double A[MAXN][MAXN], Qm[MAXN][MAXN], lam[MAXN];
    for (int a = 0; a < m; ++a)
      for (int c = 0; c < m; ++c) A[a][c] = bh.K1[a + 1][c + 1];
    jacobi_eig(m, A, Qm, lam);
    double L[MAXN] = {0};
    bool used[MAXN] = {false};
    bh.Q[0][0] = 1.0;
    for (int c = 1; c < nu; ++c) {
      // the unused eigenvector of the smallest eigenvalue among those on the modes of c's parity
      int best = -1;
      for (int k = 0; k < m; ++k) {
        if (used[k]) continue;
        double on = 0, off = 0;
        for (int a = 1; a < nu; ++a) (((a + c) & 1) ? off : on) += std::fabs(Qm[a - 1][k]);
        if (off != 0.0 || on == 0.0) continue;
        if (best < 0 || lam[k] < lam[best]) best = k;
      }
      if (best < 0) return "the 1D stiffness matrix has no eigenbasis of definite parity";
      used[best] = true;
      L[c] = lam[best];
      for (int a = 1; a < nu; ++a) bh.Q[a][c] = Qm[a - 1][best];
    }
    for (int i = 0; i < nu; ++i)
      for (int j = 0; j < nu; ++j) bh.ilam2[i][j] = (i == 0 && j == 0) ? 1.0 : 1.0 / (L[i] + L[j]);
  }
  return nullptr;
}

}  // namespace wedg
