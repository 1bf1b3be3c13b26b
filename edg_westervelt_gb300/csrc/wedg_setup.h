// Set-up kernels of wedg_create (wedg_setup.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace wedg {

// Packed inverses of the pinned c²-stiffness of every element (one block per element);
// Cw in the device layout [(r + nq s) E + e], Pu and Su column-major (nq × nu); Ainv
// [row E + e]; *bad counts the elements whose matrix is not positive definite.
__global__ void k_ainv(const double *Cw, int E, int nu, const double *Pu, const double *Su, double *Ainv,
                       unsigned int *bad);
size_t ainv_smem(int nu);   // dynamic shared memory of k_ainv

// ---- the arrays of `pre` built on the device from point values (wedg_create_points). Point
//      arrays are the reference's column-major arrays: element quantities (N, N, n, n) at
//      [e + E (r + n s)], e = j + N k; face quantities (nq, N+1, N) / (nq, N, N+1) at
//      [i + nq (jf + (N+1) k)] / [i + nq (j + N kf)].

// Flags of the constant-coefficient test (bit 0: some element's c²W or αW is not c² W or α W
// with one c², α, or c² ≤ 0) and of the faces (bit 1: c² or α jumps across a face; bit 2: a
// jump term JC is not zero)
enum { PTS_NOT_CONSTANT = 1, PTS_JUMPS = 2, PTS_JC = 4 };

// The test of src/solver.jl's element matrices for the constant-coefficient kernels, from c and α
// at the u-points: Cw = c² W, Aw = α W with W = w ⊗ w (wedg_create's test on pre's Cw, Aw)
// A coefficient at the points: an array of its values there, a constant (p and tab null), or a
// table of values on an m × n grid of cells of the unit square, row-major [row (y)][column (x)],
// looked up as the host's piecewise functions do: row = clip(floor(m y), 0, m-1), column likewise
struct PtsField {
  const double *p;
  double value;
  const double *tab;
  int m, n;
  __device__ __forceinline__ double cell(double x, double y) const {
    int r = (int)floor((double)m * y), c = (int)floor((double)n * x);
    r = r < 0 ? 0 : r > m - 1 ? m - 1 : r;
    c = c < 0 ? 0 : c > n - 1 ? n - 1 : c;
    return tab[r * n + c];
  }
  // at point i of an element array, whose coordinates are (x, y)
  __device__ __forceinline__ double at(size_t i, double x, double y) const {
    return p ? p[i] : tab ? cell(x, y) : value;
  }
};
// The coordinates of the points: the u-points of the columns (xq) and rows (yq), (N, nq), and the
// high-order points (xh, yh), (N, qh), column-major; h = 1/N
struct PtsGrid {
  const double *xq, *yq, *xh, *yh;
  int N;
  double h;
};
__global__ void k_pts_check(PtsField c_q, PtsField a_q, PtsGrid g, const double *w, int nq, int E, unsigned *flags);
// c² and α per element (and 1/c²) for the constant-coefficient kernels, or Cw, Aw in the device
// layout [(r + nq s) E + e] for the general kernels (null outputs are skipped)
__global__ void k_pts_elem(PtsField c_q, PtsField a_q, PtsGrid g, const double *w, int nq, int E, double *c2e,
                           double *ae, double *ic2e, double *Cw, double *Aw);

// One family of face values (src/solver.jl:371-408): the value at the face point and δ on either
// side, and the tolerance term s of the family; a constant family (at and tab null) is `value`
// everywhere; a table family (tab) is looked up at the face points and δ on either side
struct PtsFace {
  const double *at, *lo, *hi;
  double s, value;
  const double *tab;
  int m, n;
};
// The face arrays of `pre` in the kernels' layouts from the one-sided values of c, α, β and of the
// data derivative g0 (src/solver.jl:538-568, 716-770); horizontal when hor (face row jf, column k),
// else vertical (row j, face column kf). g0 may have null arrays (source mode: g0 = 0).
struct PtsFaceOut {
  double *c2, *af, *cf, *bf, *c2m, *afm, *JC;
};
__global__ void k_pts_faces(int N, int nq, bool hor, PtsGrid g, PtsFace c, PtsFace a, PtsFace b, PtsFace g0,
                            PtsFaceOut o, unsigned *flags);
// max |value| of a table family at the points δ off the faces inside the domain (the values
// side_values takes the tolerance term from), as the bits of the non-negative double, atomicMax
__global__ void k_pts_face_max(int N, int nq, PtsGrid g, PtsFace f, unsigned long long *out);

// The projections Π(X)[a, b] = Σ_r Σ_s P_h[r, a] W[r, s] X[r, s] P_h[s, b] of the element data
// at the high-order points (src/solver.jl:704-764), into [(a + nv b) E + e]: kind 0 X = x1,
// kind 1 X = x2 x1² (β Φ²), kind 2 the Gaussian source amplitude exp(-|x - x0|²/r0²) at the
// points (xh, yh: (N, qh) column-major local coordinates of the columns and rows).
struct PtsProj {
  int kind;
  const double *x1;
  PtsField x2;
  double amp, x0, y0, r0;
};
__global__ void k_pts_proj(PtsGrid g, int qh, int nv, const double *Ph, const double *Wh, PtsProj p, double *out);

// 2β at the high-order points, [(r + qh s) E + e]
__global__ void k_pts_beta2(PtsGrid g, int qh, PtsField b, double *out);

}  // namespace wedg
