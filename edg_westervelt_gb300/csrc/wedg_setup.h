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
// A point array, or the one value of a field that is constant (p null)
struct PtsField {
  const double *p;
  double value;
  __device__ __forceinline__ double operator[](size_t i) const { return p ? p[i] : value; }
};
__global__ void k_pts_check(PtsField c_q, PtsField a_q, const double *w, int nq, int E, unsigned *flags);
// c² and α per element (and 1/c²) for the constant-coefficient kernels, or Cw, Aw in the device
// layout [(r + nq s) E + e] for the general kernels (null outputs are skipped)
__global__ void k_pts_elem(PtsField c_q, PtsField a_q, const double *w, int nq, int E, double *c2e, double *ae,
                           double *ic2e, double *Cw, double *Aw);

// One family of face values (src/solver.jl:371-408): the value at the face point and δ on either
// side, and the tolerance term s of the family; a constant family (at null) is `value` everywhere
struct PtsFace {
  const double *at, *lo, *hi;
  double s, value;
};
// The face arrays of `pre` in the kernels' layouts from the one-sided values of c, α, β and of the
// data derivative g0 (src/solver.jl:538-568, 716-770); horizontal when hor (face row jf, column k),
// else vertical (row j, face column kf). g0 may have null arrays (source mode: g0 = 0).
struct PtsFaceOut {
  double *c2, *af, *cf, *bf, *c2m, *afm, *JC;
};
__global__ void k_pts_faces(int N, int nq, bool hor, PtsFace c, PtsFace a, PtsFace b, PtsFace g0, PtsFaceOut o,
                            unsigned *flags);

// The projections Π(X)[a, b] = Σ_r Σ_s P_h[r, a] W[r, s] X[r, s] P_h[s, b] of the element data
// at the high-order points (src/solver.jl:704-764), into [(a + nv b) E + e]: kind 0 X = x1,
// kind 1 X = x2 x1² (β Φ²), kind 2 the Gaussian source amplitude exp(-|x - x0|²/r0²) at the
// points (xh, yh: (N, qh) column-major local coordinates of the columns and rows).
struct PtsProj {
  int kind;
  const double *x1;
  PtsField x2;
  const double *xh, *yh;
  double amp, x0, y0, r0;
};
__global__ void k_pts_proj(int N, int qh, int nv, const double *Ph, const double *Wh, PtsProj p, double *out);

// y = a x elementwise
__global__ void k_pts_scale(size_t n, double a, PtsField x, double *y);

}  // namespace wedg
