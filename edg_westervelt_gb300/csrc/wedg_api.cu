// Host runtime and C ABI of libwedg (declared in include/wedg.h).
//
// wedg_create turns the reference's `pre` (host arrays in Julia layouts,
// src/solver.jl:428-770) into device arrays in element-fastest layouts,
// builds the 1D operators the kernels take as parameters, and detects the
// constant-coefficient fast path. The call functions enqueue the two kernels
// of each stage (wedg_kernels.cuh) on the workspace stream and report errors
// with the reference's semantics: boundary-weight errors before mass errors
// (src/rhs.jl:530-531), the first failing point or element in the order of the
// serial loops, and the state left untouched by a failing RK4 step.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wedg.h"
#include "wedg_basis.h"
#include "wedg_diag.h"
#include "wedg_setup.h"
#include "wedg_dispatch.h"

namespace wedg {

__global__ void k_rk4_final(int n_u, int n_v, double *u, double *v, const double *accu, const double *accv,
                            double c, const unsigned long long *err, unsigned int *nonfinite) {
  if (*(volatile const unsigned long long *)err != ERR_NONE) return;
  bool fin = true;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_u + n_v; i += gridDim.x * blockDim.x) {
    if (i < n_u) {
      const double x = u[i] + c * accu[i];
      u[i] = x;
      fin = fin && isfinite(x);
    } else {
      const int l = i - n_u;
      const double x = v[l] + c * accv[l];
      v[l] = x;
      fin = fin && isfinite(x);
    }
  }
  if (!fin) atomicOr(nonfinite, 1u);
}

__global__ void k_step_done(unsigned long long *err, const unsigned int *nonfinite, int stop_nonfinite,
                            long long *steps_done) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (*err != ERR_NONE) return;
  *steps_done += 1;
  if (stop_nonfinite && *nonfinite) *err = (3ull << ERR_CLASS_SHIFT);
}

// out = a x + b y (+ z), elementwise; y, z may be null
__global__ void k_lincomb(size_t n, double *out, double a, const double *x, double b, const double *y,
                          const double *z) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double r = a * x[i];
    if (y) r = fma(b, y[i], r);
    if (z) r += z[i];
    out[i] = r;
  }
}

// The candidates of the autotuners, tried one coordinate at a time (k_prep's block, then the
// mass solves'); a candidate replaces the best so far only when it is faster by more than 2 %
const int kTuneThreads[3] = {32, 64, 128};
constexpr double kTuneGain = 0.98;

Launchers get_launchers(int nu, int nv, bool fast) {
  switch (nu) {
    case 2: return launchers_q1(nv, fast);
    case 3: return launchers_q2(nv, fast);
    case 4: return launchers_q3(nv, fast);
    case 5: return launchers_q4(nv, fast);
    case 6: return launchers_q5(nv, fast);
    case 7: return launchers_q6(nv, fast);
    case 8: return launchers_q7(nv, fast);
    default: return Launchers();
  }
}

}  // namespace wedg

using namespace wedg;

struct wedg_ws {
  wedg_config cfg;
  int N = 0, E = 0, nu = 0, nv = 0, nq = 0, qh = 0;
  bool fast = false;
  Launchers L;
  BasisHost bh;
  std::vector<char> basis;
  Fields F{};
  cudaStream_t own_stream = nullptr, stream = nullptr;
  std::vector<void *> allocs;
  size_t bytes = 0;
  // state buffers
  double *d_u = nullptr, *d_v = nullptr, *d_ut = nullptr, *d_vt = nullptr;
  double *su = nullptr, *sv = nullptr, *accu = nullptr, *accv = nullptr;
  long long *steps_done = nullptr;
  int parity = 0;   // bin-count buffer of the next stage
  // launch shapes (set by wedg_set_launch_shape or the autotuners): threads per block of k_prep
  // (one element per thread) and of the mass solves (teams of threads per element); shape_gen
  // counts the changes, so that a captured batch graph is captured again after one
  int prep_threads = 128, mass_threads = CHEB_THREADS;
  int64_t shape_gen = 0;
  // adjoint scratch (allocated on first use): μ, ν, -(h²/4)ν, forward ut and vt, slot weights
  double *adj_mu = nullptr, *adj_nu = nullptr, *adj_nus = nullptr, *adj_ut = nullptr, *adj_vt = nullptr;
  double *adj_hat = nullptr;
  double *adj_in[4] = {nullptr, nullptr, nullptr, nullptr};   // host-call copies of u, v, λ_u, λ_v
  // reverse RK4: checkpoints, the stage states of one segment, λ, its update, K̄ and Jᵀ K̄
  std::vector<double *> rk_chk, rk_seg;
  int64_t rk_chk_n = 0, rk_seg_n = 0;
  double *rk_lam = nullptr, *rk_acc = nullptr, *rk_kbar = nullptr, *rk_g = nullptr, *rk_y = nullptr;
  double *rk_par = nullptr;   // per-element gradients with respect to c², α, β
  // the forward run the next reverse sweep differentiates
  bool rk_ready = false;
  double rk_dt = 0;
  int64_t rk_nsteps = 0, rk_every = 1;
  std::vector<double> rk_t;
  // the forward data of every stage of one segment, kept by the reverse sweep (see
  // wedg_set_adjoint_memory): the stage RHS K = (ut | vt), traces, G, Chebyshev data
  struct StageData {
    double *k = nullptr, *tr = nullptr, *G = nullptr, *th = nullptr, *de = nullptr;
    int *nst = nullptr, *bins = nullptr, *bin_count = nullptr;
    int parity = 0;
  };
  std::vector<StageData> rk_keep;
  int64_t adj_mem = -1;
  // optional per-launch timing (events recorded around each stage kernel)
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  struct EvQuad { cudaEvent_t a, b, c, d; };   // prep runs from a to b, stage from b to c, mass from c to d
  std::vector<EvQuad> ev_pending;
  double t_prep = 0, t_stage = 0, t_mass = 0;
  int64_t n_prep = 0, n_stage = 0, n_mass = 0;
  // last call
  int status = WEDG_OK;
  int64_t key = 0;
  std::string message;
  wedg_stats stats{};
};

namespace {

int cuda_fail(wedg_ws *ws, cudaError_t e, const char *what) {
  if (ws) {
    ws->status = WEDG_ERR_CUDA;
    ws->message = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  }
  return WEDG_ERR_CUDA;
}

#define CK(ws, call)                                          \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(ws, e_, #call);   \
  } while (0)

template <typename T>
int dalloc(wedg_ws *ws, T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  void *q = nullptr;
  CK(ws, cudaMalloc(&q, n * sizeof(T)));
  ws->allocs.push_back(q);
  ws->bytes += n * sizeof(T);
  *p = static_cast<T *>(q);
  return WEDG_OK;
}

template <typename T>
int upload(wedg_ws *ws, const T **dst, const std::vector<T> &h) {
  T *p;
  int rc = dalloc(ws, &p, h.size());
  if (rc) return rc;
  CK(ws, cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  *dst = p;
  return WEDG_OK;
}

const char *kind_name(int k) {
  switch (k) {
    case WEDG_ABSORBING_2BETA: return "absorbing_2beta";
    case WEDG_ABSORBING: return "absorbing";
    case WEDG_DIRICHLET: return "dirichlet";
    case WEDG_WALL: return "wall";
    default: return "?";
  }
}

// Julia's `string(x)` for the tolerance in the CG warning (1.0e-14 style)
std::string julia_float(double x) {
  char buf[64];
  for (int p = 1; p <= 17; ++p) {
    snprintf(buf, sizeof buf, "%.*e", p - 1, x);
    if (std::strtod(buf, nullptr) == x) break;
  }
  std::string s(buf);
  const size_t epos = s.find('e');
  std::string mant = s.substr(0, epos);
  int ex = std::atoi(s.c_str() + epos + 1);
  if (ex >= -5 && ex < 16) {
    snprintf(buf, sizeof buf, "%.17g", x);
    std::string t;
    for (int p = 1; p <= 17; ++p) {
      snprintf(buf, sizeof buf, "%.*g", p, x);
      if (std::strtod(buf, nullptr) == x) break;
    }
    t = buf;
    if (t.find('.') == std::string::npos && t.find('e') == std::string::npos) t += ".0";
    return t;
  }
  if (mant.find('.') == std::string::npos) mant += ".0";
  return mant + "e" + std::to_string(ex);
}

// shape check of src/rhs.jl:500-503
int check_shapes(wedg_ws *ws, const int64_t *us, const int64_t *vs) {
  const int N = ws->N;
  bool ok = us && vs && us[0] == N && us[1] == N && us[2] == ws->nu && us[3] == ws->nu && vs[0] == N &&
            vs[1] == N && vs[2] == ws->nv && vs[3] == ws->nv;
  if (ok) return WEDG_OK;
  ws->status = WEDG_ERR_DIMENSION;
  ws->message = "state, workspace and pre do not match (N = " + std::to_string(N) +
                ", q_u + 1 = " + std::to_string(ws->nu) + ", q_v + 1 = " + std::to_string(ws->nv) + ")";
  return WEDG_ERR_DIMENSION;
}

void stage_factors(const wedg_ws *ws, double t, StageIO &S) {
  const wedg_config &c = ws->cfg;
  const double om = c.omega;
  S.ct = c.mms_on ? std::cos(om * t) : 0.0;
  S.st = c.mms_on ? std::sin(om * t) : 0.0;
  S.srct = 0.0;
  if (c.src_on && t < c.src_Ts) {
    const double s = std::sin(M_PI * t / c.src_Ts);
    S.srct = std::sin(c.src_omega * t) * (s * s);
  }
  S.cSP = -(om * om) * S.ct;
  S.cB = -2.0 * (om * om * om) * S.st * S.ct;
  S.cC = 1.0 - S.ct;
  S.cD = om * S.st;
}

int reset_flags(wedg_ws *ws) {
  CK(ws, cudaMemsetAsync(ws->F.err, 0xFF, sizeof(unsigned long long), ws->stream));
  CK(ws, cudaMemsetAsync(ws->F.cg_nfail, 0, sizeof(unsigned int), ws->stream));
  CK(ws, cudaMemsetAsync(ws->F.nonfinite, 0, sizeof(unsigned int), ws->stream));
  CK(ws, cudaMemsetAsync(ws->F.nmax, 0, sizeof(int), ws->stream));
  CK(ws, cudaMemsetAsync(ws->F.nsum, 0, sizeof(unsigned long long), ws->stream));
  CK(ws, cudaMemsetAsync(ws->F.bin_count, 0, 2 * NBIN * sizeof(int), ws->stream));
  ws->parity = 0;
  ws->stats.element_stages = 0;
  CK(ws, cudaMemsetAsync(ws->steps_done, 0, sizeof(long long), ws->stream));
  return WEDG_OK;
}

cudaEvent_t take_event(wedg_ws *ws) {
  if (!ws->ev_pool.empty()) {
    cudaEvent_t e = ws->ev_pool.back();
    ws->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// fold the recorded launch durations into the totals (after a synchronization)
void drain_events(wedg_ws *ws) {
  for (auto &p : ws->ev_pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) { ws->t_prep += ms; ws->n_prep += 1; }
    if (cudaEventElapsedTime(&ms, p.b, p.c) == cudaSuccess) { ws->t_stage += ms; ws->n_stage += 1; }
    if (cudaEventElapsedTime(&ms, p.c, p.d) == cudaSuccess) { ws->t_mass += ms; ws->n_mass += 1; }
    ws->ev_pool.push_back(p.a);
    ws->ev_pool.push_back(p.b);
    ws->ev_pool.push_back(p.c);
    ws->ev_pool.push_back(p.d);
  }
  ws->ev_pending.clear();
}

// enqueue the three kernels of one stage (on the workspace's Fields, or on Fo)
int enqueue_stage(wedg_ws *ws, const StageIO &S, const Fields *Fo = nullptr) {
  const Fields &F = Fo ? *Fo : ws->F;
  const int tp = ws->prep_threads, bp = (ws->E + tp - 1) / tp;
  const int ts = stage_threads(ws->nu, ws->nv, ws->fast), bs = (ws->E + ts - 1) / ts;
  const int bm = 1;   // the mass kernels size their own grid
  StageIO Sp = S;
  Sp.parity = ws->parity;
  ws->parity = 1 - ws->parity;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
  if (ws->timing) {
    e0 = take_event(ws); e1 = take_event(ws); e2 = take_event(ws); e3 = take_event(ws);
    cudaEventRecord(e0, ws->stream);
  }
  ws->L.prep(ws->basis.data(), F, Sp, bp, tp, ws->stream);
  if (ws->timing) cudaEventRecord(e1, ws->stream);
  ws->L.stage(ws->basis.data(), F, Sp, bs, ts, ws->stream);
  if (ws->timing) cudaEventRecord(e2, ws->stream);
  ws->L.mass(ws->basis.data(), F, Sp, bm, ws->mass_threads, ws->stream);
  if (ws->timing) {
    cudaEventRecord(e3, ws->stream);
    ws->ev_pending.push_back({e0, e1, e2, e3});
  }
  ws->stats.kernel_launches += 3;
  ws->stats.element_stages += ws->E;
  CK(ws, cudaGetLastError());
  return WEDG_OK;
}

// one RK4 step on device state u, v (src/solver.jl:289-297)
// Time factors of the four stages of `count` steps from the step at time t (t advancing by
// t += dt), 8 doubles per stage (the seven of StageIO and a pad), for graph replays.
void factor_table(const wedg_ws *ws, double t, double dt, int64_t count, double *out) {
  for (int64_t it = 0; it < count; ++it) {
    const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
    for (int s = 0; s < 4; ++s) {
      StageIO S{};
      stage_factors(ws, ts[s], S);
      double *f = out + (it * 4 + s) * 8;
      f[0] = S.ct; f[1] = S.st; f[2] = S.srct; f[3] = S.cSP; f[4] = S.cB; f[5] = S.cC; f[6] = S.cD; f[7] = 0.0;
    }
    t += dt;
  }
}

// One RK4 step on the workspace stream. With tf != nullptr the stage kernels take their time
// factors from the device table tf (tf_n steps, indexed by the device step counter), so that the
// launches can be captured once into a CUDA graph and replayed for every step.
int enqueue_rk4(wedg_ws *ws, double *u, double *v, double t, double dt, int stop_nonfinite,
                const double *tf = nullptr, long long tf_n = 0, double *const *stage_u = nullptr,
                double *const *stage_v = nullptr) {
  // with stage_u, stage_v (four buffers each) the stage states Y1..Y4 of the step are kept there
  const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
  const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
  const bool cg = ws->cfg.mass_solver == WEDG_CG;
  if (stage_u) {
    const size_t bU = sizeof(double) * ws->E * ws->nu * ws->nu, bV = sizeof(double) * ws->E * ws->nv * ws->nv;
    CK(ws, cudaMemcpyAsync(stage_u[0], u, bU, cudaMemcpyDeviceToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(stage_v[0], v, bV, cudaMemcpyDeviceToDevice, ws->stream));
  }
  for (int s = 0; s < 4; ++s) {
    StageIO S{};
    S.xu = s == 0 ? u : (stage_u ? stage_u[s] : ws->su);
    S.xv = s == 0 ? v : (stage_v ? stage_v[s] : ws->sv);
    if (tf) {
      S.tf = tf;
      S.tf_n = tf_n;
      S.step = ws->steps_done;
      S.stage = s;
    } else {
      stage_factors(ws, ts[s], S);
    }
    S.u0 = u; S.v0 = v;
    S.su = stage_u && s < 3 ? stage_u[s + 1] : ws->su;
    S.sv = stage_v && s < 3 ? stage_v[s + 1] : ws->sv;
    S.accu = ws->accu; S.accv = ws->accv;
    S.uo = u; S.vo = v;
    if (s < 3) {
      S.mode = OUT_RK4_STAGE;
      S.first = s == 0;
      S.c = cs[s];
    } else {
      S.mode = cg ? OUT_RK4_LAST_ACC : OUT_RK4_LAST;
      S.c = dt / 6.0;
    }
    int rc = enqueue_stage(ws, S);
    if (rc) return rc;
  }
  if (cg) {
    const int nU = ws->E * ws->nu * ws->nu, nV = ws->E * ws->nv * ws->nv;
    const int blocks = std::min((nU + nV + 255) / 256, 152 * 8);
    k_rk4_final<<<blocks, 256, 0, ws->stream>>>(nU, nV, u, v, ws->accu, ws->accv, dt / 6.0, ws->F.err,
                                                ws->F.nonfinite);
    ws->stats.kernel_launches += 1;
  }
  k_step_done<<<1, 32, 0, ws->stream>>>(ws->F.err, ws->F.nonfinite, stop_nonfinite, ws->steps_done);
  ws->stats.kernel_launches += 1;
  CK(ws, cudaGetLastError());
  return WEDG_OK;
}

// read the flags after a synchronized call and turn them into the status
int adjoint_buffers(wedg_ws *ws) {
  if (ws->adj_mu) return WEDG_OK;
  const size_t nU = (size_t)ws->E * ws->nu * ws->nu, nV = (size_t)ws->E * ws->nv * ws->nv;
  int rc;
  if ((rc = dalloc(ws, &ws->adj_nu, nU)) || (rc = dalloc(ws, &ws->adj_nus, nU)) || (rc = dalloc(ws, &ws->adj_ut, nU)) ||
      (rc = dalloc(ws, &ws->adj_vt, nV)) || (rc = dalloc(ws, &ws->adj_hat, (size_t)3 * 4 * ws->nq * ws->E)) ||
      (rc = dalloc(ws, &ws->adj_in[0], nU)) || (rc = dalloc(ws, &ws->adj_in[1], nV)) ||
      (rc = dalloc(ws, &ws->adj_in[2], nU)) || (rc = dalloc(ws, &ws->adj_in[3], nV)) ||
      (rc = dalloc(ws, &ws->adj_mu, nV)))
    return rc;
  return WEDG_OK;
}

// The transpose of one RHS evaluation on the workspace stream (see wedg_adjoint.cuh for the
// steps), after the forward evaluation at the state: Fs holds its traces and Chebyshev data, S
// the state (xu, xv), its time factors and bin parity and the forward outputs (ut, vt). Writes
// Jᵀ(λ_u, λ_v) to (gu, gv); with gpar (3E: c², α, β), the derivatives of λ·RHS with respect to
// the per-element coefficients are added to it.
int enqueue_adjoint_core(wedg_ws *ws, const Fields &Fs, const StageIO &S, const double *lam_u, const double *lam_v,
                         double *gu, double *gv, double *gpar) {
  const int ts = stage_threads(ws->nu, ws->nv, ws->fast), bs = (ws->E + ts - 1) / ts;
  // μ = M(v)⁻¹ λ_v, on the Chebyshev data of the state
  Fields Fm = Fs;
  Fm.mrhs = const_cast<double *>(lam_v);
  StageIO Sm = S;
  Sm.mode = OUT_RHS;
  Sm.vt = ws->adj_mu;
  ws->L.mass(ws->basis.data(), Fm, Sm, 1, ws->mass_threads, ws->stream);
  // ν = A_e⁻¹ λ_u
  StageIO Su = S;
  Su.mode = OUT_ADJ_USOLVE;
  Su.xu = lam_u;
  Su.ut = ws->adj_nu;
  ws->L.stage(ws->basis.data(), Fs, Su, bs, ts, ws->stream);
  const AdjIO A{ws->adj_mu, ws->adj_nu, ws->adj_nus, S.vt, ws->adj_hat, gu, gv, S.xv,
                gpar ? gpar + 2 * (size_t)ws->E : nullptr};
  ws->L.adj_hats(ws->basis.data(), Fs, S, A, ws->stream);
  // the volume transposes: the volume terms of the state (-(h²/4) ν, μ)
  StageIO Sv = S;
  Sv.mode = OUT_ADJ_VOLUME;
  Sv.xu = ws->adj_nus;
  Sv.xv = ws->adj_mu;
  Sv.vt = gv;
  Sv.ut = gu;
  ws->L.stage(ws->basis.data(), Fs, Sv, bs, ts, ws->stream);
  ws->L.adj_mass(ws->basis.data(), Fs, S, A, ws->stream);
  // the faces; with gpar also K̄·∂F/∂p at the state: volume, u-solve and faces (the mass
  // matrix's β-part is in k_adj_mass)
  ws->L.adj_face(ws->basis.data(), Fs, S, A, gpar, gpar ? gpar + ws->E : nullptr,
                 gpar ? gpar + 2 * (size_t)ws->E : nullptr, ws->stream);
  ws->stats.kernel_launches += 6;
  CK(ws, cudaGetLastError());
  return WEDG_OK;
}

// Jᵀ(λ_u, λ_v) of the RHS at the state (u, v), time t, into (gu, gv); device pointers: the
// forward RHS at the state first (its traces, Chebyshev data and vt are inputs of the
// transpose), then the transpose.
int enqueue_rhs_adjoint(wedg_ws *ws, const double *u, const double *v, double t, const double *lam_u,
                        const double *lam_v, double *gu, double *gv, double *gpar = nullptr) {
  int rc = adjoint_buffers(ws);
  if (rc) return rc;
  StageIO S{};
  S.xu = u; S.xv = v;
  stage_factors(ws, t, S);
  S.mode = OUT_RHS;
  S.ut = ws->adj_ut;
  S.vt = ws->adj_vt;
  const int par = ws->parity;
  if ((rc = enqueue_stage(ws, S))) return rc;
  S.parity = par;
  return enqueue_adjoint_core(ws, ws->F, S, lam_u, lam_v, gu, gv, gpar);
}

// The workspace's Fields with the per-stage arrays of kept stage data d
Fields kept_fields(const wedg_ws *ws, const wedg_ws::StageData &d) {
  Fields F = ws->F;
  F.tr = d.tr; F.G = d.G; F.th = d.th; F.de = d.de;
  F.nst = d.nst; F.bins = d.bins; F.bin_count = d.bin_count;
  return F;
}

// bytes of the kept data of one stage
size_t stage_data_bytes(const wedg_ws *ws) {
  const size_t E = ws->E;
  return sizeof(double) * E * ((size_t)ws->nu * ws->nu + ws->nv * ws->nv + 12 * ws->nq + ws->qh * ws->qh + 2) +
         sizeof(int) * (E * (1 + NBIN) + 2 * NBIN);
}

int collect(wedg_ws *ws) {
  unsigned long long err;
  unsigned int cgf, nonf;
  int nmax;
  long long done;
  unsigned long long nsum;
  CK(ws, cudaStreamSynchronize(ws->stream));
  drain_events(ws);
  CK(ws, cudaMemcpy(&nsum, ws->F.nsum, sizeof nsum, cudaMemcpyDeviceToHost));
  ws->stats.cheb_steps_sum = (int64_t)nsum;
  CK(ws, cudaMemcpy(&err, ws->F.err, sizeof err, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(&cgf, ws->F.cg_nfail, sizeof cgf, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(&nonf, ws->F.nonfinite, sizeof nonf, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(&nmax, ws->F.nmax, sizeof nmax, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(&done, ws->steps_done, sizeof done, cudaMemcpyDeviceToHost));
  ws->stats.cg_not_converged = (int32_t)cgf;
  ws->stats.finite = nonf ? 0 : 1;
  ws->stats.cheb_steps_max = nmax;
  ws->stats.steps_done = done;
  ws->status = WEDG_OK;
  ws->key = 0;
  ws->message.clear();
  if (err != ERR_NONE) {
    const unsigned cls = (unsigned)(err >> ERR_CLASS_SHIFT);
    const int64_t key = (int64_t)(err & ((1ull << ERR_CLASS_SHIFT) - 1));
    if (cls == 0) {
      // src/rhs.jl:768-776 and :112-116
      const int s = (int)((key - 1) / (2 * (int64_t)ws->nq * ws->N));
      const int check = (key % 2 == 1) ? 1 : 2;
      const std::string kk = ws->cfg.kb[s] == 2.0 ? "2" : "";
      const std::string kind = kind_name(ws->cfg.kind[s]);
      ws->status = WEDG_ERR_BOUNDARY_WEIGHT;
      ws->key = key;
      ws->message = check == 1 ? "boundary weight 1 - " + kk + "βv_h ≤ 0 at a face point (" + kind + " side)"
                               : "boundary weight 1 - " + kk + "βg ≤ 0 for the boundary data g (" + kind + " side)";
    } else if (cls == 1) {
      ws->status = WEDG_ERR_MASS_NOT_PD;
      ws->key = key;
      if (ws->cfg.mass_solver == WEDG_CG) {
        const int64_t j = (key - 1) % ws->N + 1, k = (key - 1) / ws->N + 1;
        ws->message = "mass matrix not positive definite on element (" + std::to_string(j) + ", " +
                      std::to_string(k) + "): 1 - 2βv_h ≤ 0";
      } else {
        ws->message = "mass matrix not positive definite on element " + std::to_string(key) + ": 1 - 2βv_h ≤ 0";
      }
    }
    // class 3: a run stopped after a non-finite step; not an error of the call
  }
  if (ws->status == WEDG_OK && cgf > 0 && ws->cfg.mass_solver == WEDG_CG) {
    ws->status = WEDG_WARN_CG_NOT_CONVERGED;
    ws->message = "mass solve: " + std::to_string(cgf) + " element systems did not reach the tolerance " +
                  julia_float(ws->cfg.mass_tol);
  }
  return ws->status;
}

int argument_error(wedg_ws *ws, const std::string &msg) {
  if (ws) {
    ws->status = WEDG_ERR_ARGUMENT;
    ws->message = msg;
  }
  return WEDG_ERR_ARGUMENT;
}

}  // namespace

namespace {

// Device buffers of one wedg_run_source call, freed (after the stream is idle) on every return path.
struct RunBuffers {
  cudaStream_t st = nullptr;
  std::vector<void *> p;
  template <typename T>
  cudaError_t get(T **q, size_t n) {
    *q = nullptr;
    void *x = nullptr;
    const cudaError_t e = cudaMalloc(&x, (n ? n : 1) * sizeof(T));
    if (e == cudaSuccess) { p.push_back(x); *q = static_cast<T *>(x); }
    return e;
  }
  ~RunBuffers() {
    if (st) cudaStreamSynchronize(st);
    for (void *x : p) cudaFree(x);
  }
};

}  // namespace

// A batch of workspaces advanced by one replayed CUDA graph per step (wedg_batch_*)
struct wedg_batch {
  std::vector<wedg_ws *> ws;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaEvent_t half_done[2] = {nullptr, nullptr};   // the host half of the tables may be refilled
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // what the captured graph was made for
  std::vector<double *> gu, gv;
  std::vector<double> gdt;
  std::vector<int64_t> gshape;   // the instances' shape_gen
  int gstop = -1;
  // per instance: device factor table of 2 chunks (the kernels index it by step mod 2 chunks)
  std::vector<double *> d_tf;
  double *h_tf = nullptr;                           // pinned: 2 halves × instances × one chunk
  ~wedg_batch() {
    if (main) cudaStreamSynchronize(main);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (double *p : d_tf) cudaFree(p);
    if (h_tf) cudaFreeHost(h_tf);
    for (cudaEvent_t e : join) cudaEventDestroy(e);
    for (cudaEvent_t e : half_done)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (main) cudaStreamDestroy(main);
  }
};

extern "C" {

int wedg_create(const wedg_config *cfg, const wedg_pre *pre, wedg_ws **out) {
  if (!out) return WEDG_ERR_ARGUMENT;
  *out = nullptr;
  if (!cfg || !pre) return WEDG_ERR_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return WEDG_ERR_NO_DEVICE;
  const int N = cfg->N, nu = cfg->qu1, nv = cfg->qv1;
  if (N < 1 || nu < 2 || nu > MAXN || !(nv == nu || nv == nu - 1) || cfg->q_high != qhigh(nu, nv))
    return WEDG_ERR_ARGUMENT;
  if ((int64_t)N * N > (int64_t)1 << 30) return WEDG_ERR_ARGUMENT;
  for (int s = 0; s < 4; ++s)
    if (cfg->kind[s] < 0 || cfg->kind[s] > 3) return WEDG_ERR_ARGUMENT;
  if (cfg->mass_solver != WEDG_CHEBYSHEV && cfg->mass_solver != WEDG_CG) return WEDG_ERR_ARGUMENT;
  const double *need[] = {pre->w, pre->P_u, pre->S_u, pre->Ebl_u, pre->Ebr_u, pre->E1bl_u, pre->E1br_u,
                          pre->P_h_v, pre->W2d_h, pre->Cw, pre->Aw, pre->hc2, pre->haf, pre->hcf, pre->hbf,
                          pre->vc2, pre->vaf, pre->vcf, pre->vbf, pre->hc2m, pre->hafm, pre->vc2m, pre->vafm,
                          pre->hJC, pre->vJC, pre->bcB_sp, pre->bcB_spy, pre->bcT_sp, pre->bcT_spy, pre->bcL_sp,
                          pre->bcL_spx, pre->bcR_sp, pre->bcR_spx, pre->PiSP, pre->PiBSP2, pre->PiCdiv,
                          pre->PiDdiv, pre->src_projE, pre->beta_hq};
  for (const double *p : need)
    if (!p) return WEDG_ERR_ARGUMENT;

  wedg_ws *ws = new wedg_ws();
  ws->cfg = *cfg;
  ws->N = N;
  ws->E = N * N;
  ws->nu = nu;
  ws->nv = nv;
  ws->nq = nu;
  ws->qh = cfg->q_high;
  const int E = ws->E, nq = nu, qh = ws->qh;
  const size_t Es = (size_t)E;

  // ---- 1D operators (Julia column-major inputs), with their mirror parities made exact
  BasisHost &bh = ws->bh;
  if (build_basis(cfg, pre, bh)) {
    delete ws;
    return WEDG_ERR_ARGUMENT;
  }

  // ---- constant coefficients per element? Cw = c² W and Aw = α W to 1e-14 (relative)
  std::vector<double> c2e(E), ae(E), ic2e(E);
  bool fast = !cfg->general_only;
  for (int e = 0; e < E && fast; ++e) {
    const double w00 = bh.w[0] * bh.w[0];
    const double c2 = pre->Cw[0 + nq * ((size_t)e + Es * 0)] / w00;
    const double al = pre->Aw[0 + nq * ((size_t)e + Es * 0)] / w00;
    for (int s = 0; s < nq && fast; ++s)
      for (int r = 0; r < nq; ++r) {
        const double W = bh.w[r] * bh.w[s];
        const double cw = pre->Cw[r + nq * ((size_t)e + Es * s)], aw = pre->Aw[r + nq * ((size_t)e + Es * s)];
        if (std::fabs(cw - c2 * W) > 1e-14 * std::fabs(cw) || std::fabs(aw - al * W) > 1e-14 * std::fabs(aw) ||
            !(c2 > 0)) {
          fast = false;
          break;
        }
      }
    c2e[e] = c2;
    ae[e] = al;
    ic2e[e] = 1.0 / c2;
  }
  ws->fast = fast;
  ws->L = get_launchers(nu, nv, fast);
  if (!ws->L.prep) {
    delete ws;
    return WEDG_ERR_ARGUMENT;
  }
  ws->basis.resize(ws->L.basis_size);
  ws->L.pack(bh, ws->basis.data());

  int rc = WEDG_OK;
#define UP(dst, vec)                     \
  do {                                   \
    rc = upload(ws, &(dst), vec);        \
    if (rc) { wedg_destroy(ws); return rc; } \
  } while (0)
  Fields &F = ws->F;
  F.N = N;
  F.E = E;
  // ---- element arrays, element index fastest
  if (fast) {
    UP(F.c2e, c2e);
    UP(F.ae, ae);
    UP(F.ic2e, ic2e);
  } else {
    std::vector<double> cw((size_t)nq * nq * E), aw((size_t)nq * nq * E);
    for (int s = 0; s < nq; ++s)
      for (int r = 0; r < nq; ++r)
        for (int e = 0; e < E; ++e) {
          cw[(r + nq * s) * Es + e] = pre->Cw[r + nq * ((size_t)e + Es * s)];
          aw[(r + nq * s) * Es + e] = pre->Aw[r + nq * ((size_t)e + Es * s)];
        }
    UP(F.Cw, cw);
    UP(F.Aw, aw);
    const size_t nt = (size_t)nu * nu * (nu * nu + 1) / 2;
    if (pre->Ainv_u) {
      std::vector<double> ai(nt * E);
      for (int e = 0; e < E; ++e)
        for (size_t row = 0; row < nt; ++row) ai[row * Es + e] = pre->Ainv_u[row + nt * e];
      UP(F.Ainv, ai);
    } else {
      // the packed inverses of src/solver.jl:528-535, computed on the device from Cw
      const double *Pu = nullptr, *Su = nullptr;
      UP(Pu, std::vector<double>(pre->P_u, pre->P_u + (size_t)nq * nu));
      UP(Su, std::vector<double>(pre->S_u, pre->S_u + (size_t)nq * nu));
      double *ainv = nullptr;
      unsigned int *bad = nullptr;
      if ((rc = dalloc(ws, &ainv, nt * E)) || (rc = dalloc(ws, &bad, 1))) {
        wedg_destroy(ws);
        return rc;
      }
      const size_t sm = ainv_smem(nu);
      unsigned int nbad = 0;
      cudaError_t ce = cudaMemset(bad, 0, sizeof(unsigned int));
      if (ce == cudaSuccess) ce = cudaFuncSetAttribute(k_ainv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (ce == cudaSuccess) {
        k_ainv<<<E, 128, sm>>>(F.Cw, E, nu, Pu, Su, ainv, bad);
        ce = cudaGetLastError();
      }
      if (ce == cudaSuccess) ce = cudaMemcpy(&nbad, bad, sizeof nbad, cudaMemcpyDeviceToHost);
      if (ce != cudaSuccess || nbad) {
        wedg_destroy(ws);
        return ce != cudaSuccess ? WEDG_ERR_CUDA : WEDG_ERR_ARGUMENT;
      }
      F.Ainv = ainv;
    }
  }
  // ---- face arrays: (nq, N+1, N) -> [jf + (N+1)(k + N i)], (nq, N, N+1) -> [j + N (kf + (N+1) i)]
  auto hf = [&](const double *a) {
    std::vector<double> o((size_t)nq * (N + 1) * N);
    for (int k = 0; k < N; ++k)
      for (int jf = 0; jf <= N; ++jf)
        for (int i = 0; i < nq; ++i) o[jf + (size_t)(N + 1) * (k + (size_t)N * i)] = a[i + nq * (jf + (size_t)(N + 1) * k)];
    return o;
  };
  auto vf = [&](const double *a) {
    std::vector<double> o((size_t)nq * N * (N + 1));
    for (int kf = 0; kf <= N; ++kf)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < nq; ++i) o[j + (size_t)N * (kf + (size_t)(N + 1) * i)] = a[i + nq * (j + (size_t)N * kf)];
    return o;
  };
  UP(F.hc2, hf(pre->hc2)); UP(F.haf, hf(pre->haf)); UP(F.hcf, hf(pre->hcf)); UP(F.hbf, hf(pre->hbf));
  UP(F.hc2m, hf(pre->hc2m)); UP(F.hafm, hf(pre->hafm)); UP(F.hJC, hf(pre->hJC));
  UP(F.vc2, vf(pre->vc2)); UP(F.vaf, vf(pre->vaf)); UP(F.vcf, vf(pre->vcf)); UP(F.vbf, vf(pre->vbf));
  UP(F.vc2m, vf(pre->vc2m)); UP(F.vafm, vf(pre->vafm)); UP(F.vJC, vf(pre->vJC));
  // boundary data (nq, N) -> [m + N i]
  auto bd = [&](const double *a) {
    std::vector<double> o((size_t)nq * N);
    for (int m = 0; m < N; ++m)
      for (int i = 0; i < nq; ++i) o[m + (size_t)N * i] = a[i + nq * m];
    return o;
  };
  const double *sp[4] = {pre->bcB_sp, pre->bcT_sp, pre->bcL_sp, pre->bcR_sp};
  const double *spn[4] = {pre->bcB_spy, pre->bcT_spy, pre->bcL_spx, pre->bcR_spx};
  for (int s = 0; s < 4; ++s) {
    UP(F.bsp[s], bd(sp[s]));
    UP(F.bspn[s], bd(spn[s]));
  }
  // projections (nv, nv, N, N) -> [(a + nv b) E + e]
  auto pj = [&](const double *a) {
    std::vector<double> o((size_t)nv * nv * E);
    for (int e = 0; e < E; ++e)
      for (int l = 0; l < nv * nv; ++l) o[l * Es + e] = a[l + (size_t)nv * nv * e];
    return o;
  };
  if (cfg->mms_on) {
    UP(F.PiSP, pj(pre->PiSP)); UP(F.PiBSP2, pj(pre->PiBSP2)); UP(F.PiDdiv, pj(pre->PiDdiv));
  }
  if (!cfg->src_on) UP(F.PiCdiv, pj(pre->PiCdiv));
  if (cfg->src_on) UP(F.srcP, pj(pre->src_projE));
  // β at the high-order points (qh, E, qh) -> [(r + qh s) E + e]
  {
    std::vector<double> o((size_t)qh * qh * E);
    for (int s = 0; s < qh; ++s)
      for (int e = 0; e < E; ++e)
        for (int r = 0; r < qh; ++r) o[(r + qh * s) * Es + e] = 2.0 * pre->beta_hq[r + qh * ((size_t)e + Es * s)];
    UP(F.beta2, o);
  }
#undef UP
  // ---- scratch
  const size_t nU = (size_t)nu * nu * E, nV = (size_t)nv * nv * E;
  if ((rc = dalloc(ws, &F.tr, (size_t)12 * nq * E)) || (rc = dalloc(ws, &F.G, (size_t)qh * qh * E)) ||
      (rc = dalloc(ws, &F.th, Es)) || (rc = dalloc(ws, &F.de, Es)) || (rc = dalloc(ws, &F.nst, Es)) ||
      (rc = dalloc(ws, &F.nmax, 1)) || (rc = dalloc(ws, &F.nsum, 1)) || (rc = dalloc(ws, &F.err, 1)) ||
      (rc = dalloc(ws, &F.cg_nfail, 1)) ||
      (rc = dalloc(ws, &F.nonfinite, 1)) || (rc = dalloc(ws, &ws->steps_done, 1)) ||
      (rc = dalloc(ws, &ws->d_u, nU)) || (rc = dalloc(ws, &ws->d_v, nV)) || (rc = dalloc(ws, &ws->d_ut, nU)) ||
      (rc = dalloc(ws, &ws->d_vt, nV)) || (rc = dalloc(ws, &ws->su, nU)) || (rc = dalloc(ws, &ws->sv, nV)) ||
      (rc = dalloc(ws, &ws->accu, nU)) || (rc = dalloc(ws, &ws->accv, nV)) || (rc = dalloc(ws, &F.mrhs, nV)) ||
      (rc = dalloc(ws, &F.bins, (size_t)NBIN * E)) || (rc = dalloc(ws, &F.bin_count, (size_t)2 * NBIN))) {
    wedg_destroy(ws);
    return rc;
  }
  F.theta = cfg->theta; F.tau = cfg->tau; F.lu = cfg->lambda_u; F.lv = cfg->lambda_v;
  F.omega = cfg->omega;
  const double h = 1.0 / N;
  F.two_h = 2.0 / h;
  F.four_hh = 4.0 / (h * h);
  F.mass_tol = cfg->mass_tol;
  F.Lcheb = std::acosh(1.0 / cfg->mass_tol);
  F.one_sided = cfg->one_sided ? 1 : 0;
  F.mms_on = cfg->mms_on ? 1 : 0;
  F.src_on = cfg->src_on ? 1 : 0;
  F.cg = cfg->mass_solver == WEDG_CG;
  F.cheb_common = cfg->cheb_steps == WEDG_CHEB_COMMON_MAX;
  F.sorted = !F.cg && !F.cheb_common;
  for (int s = 0; s < 4; ++s) {
    F.kind[s] = cfg->kind[s];
    F.gam[s] = cfg->gamma_abc[s]; F.eta[s] = cfg->eta_abc[s]; F.sig[s] = cfg->sigma[s];
    F.kb[s] = cfg->kb[s]; F.kap[s] = cfg->kappa[s];
  }
  // sets the shared-memory attributes of k_stage and k_cg (a launch of zero blocks does nothing else)
  ws->L.stage(ws->basis.data(), F, StageIO{}, 0, 0, nullptr);
  ws->L.mass(ws->basis.data(), F, StageIO{}, 0, 0, nullptr);
  cudaMemset(F.bin_count, 0, 2 * NBIN * sizeof(int));
  cudaError_t ce = cudaStreamCreateWithFlags(&ws->own_stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    int r = cuda_fail(ws, ce, "cudaStreamCreate");
    wedg_destroy(ws);
    return r;
  }
  ws->stream = ws->own_stream;
  ws->stats.fast_path = fast ? 1 : 0;
  ws->stats.device_bytes = (int64_t)ws->bytes;
  cudaDeviceSynchronize();
  *out = ws;
  return WEDG_OK;
}

void wedg_destroy(wedg_ws *ws) {
  if (!ws) return;
  if (ws->own_stream) cudaStreamSynchronize(ws->own_stream);
  if (ws->stream) cudaStreamSynchronize(ws->stream);
  drain_events(ws);
  for (cudaEvent_t e : ws->ev_pool) cudaEventDestroy(e);
  for (void *p : ws->allocs) cudaFree(p);
  if (ws->own_stream) cudaStreamDestroy(ws->own_stream);
  delete ws;
}

int wedg_rhs(wedg_ws *ws, const double *u, const double *v, double t, double *ut, double *vt,
             const int64_t u_shape[4], const int64_t v_shape[4], int where) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stats.kernel_launches = 0;
  int rc = check_shapes(ws, u_shape, v_shape);
  if (rc) return rc;
  if (!u || !v || !ut || !vt) return argument_error(ws, "null state pointer");
  const size_t bU = sizeof(double) * ws->E * ws->nu * ws->nu, bV = sizeof(double) * ws->E * ws->nv * ws->nv;
  const double *xu = u, *xv = v;
  double *ou = ut, *ov = vt;
  if (where == WEDG_HOST) {
    CK(ws, cudaMemcpyAsync(ws->d_u, u, bU, cudaMemcpyHostToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(ws->d_v, v, bV, cudaMemcpyHostToDevice, ws->stream));
    xu = ws->d_u; xv = ws->d_v; ou = ws->d_ut; ov = ws->d_vt;
  }
  if ((rc = reset_flags(ws))) return rc;
  StageIO S{};
  S.xu = xu; S.xv = xv;
  stage_factors(ws, t, S);
  S.mode = OUT_RHS;
  S.ut = ou; S.vt = ov;
  if ((rc = enqueue_stage(ws, S))) return rc;
  rc = collect(ws);
  if ((rc == WEDG_OK || rc == WEDG_WARN_CG_NOT_CONVERGED) && where == WEDG_HOST) {
    CK(ws, cudaMemcpy(ut, ws->d_ut, bU, cudaMemcpyDeviceToHost));
    CK(ws, cudaMemcpy(vt, ws->d_vt, bV, cudaMemcpyDeviceToHost));
  }
  return rc;
}

int wedg_rk4_steps(wedg_ws *ws, double *u, double *v, double t0, double dt, int64_t nsteps,
                   const int64_t u_shape[4], const int64_t v_shape[4], int where, int stop_nonfinite,
                   int64_t *steps_done, int *finite) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stats.kernel_launches = 0;
  int rc = check_shapes(ws, u_shape, v_shape);
  if (rc) return rc;
  if (!u || !v) return argument_error(ws, "null state pointer");
  if (nsteps < 0) return argument_error(ws, "nsteps must be ≥ 0");
  const size_t bU = sizeof(double) * ws->E * ws->nu * ws->nu, bV = sizeof(double) * ws->E * ws->nv * ws->nv;
  double *du = u, *dv = v;
  if (where == WEDG_HOST) {
    CK(ws, cudaMemcpyAsync(ws->d_u, u, bU, cudaMemcpyHostToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(ws->d_v, v, bV, cudaMemcpyHostToDevice, ws->stream));
    du = ws->d_u; dv = ws->d_v;
  }
  if ((rc = reset_flags(ws))) return rc;
  double t = t0;
  for (int64_t it = 0; it < nsteps; ++it) {
    if ((rc = enqueue_rk4(ws, du, dv, t, dt, stop_nonfinite))) return rc;
    t += dt;
  }
  rc = collect(ws);
  if (steps_done) *steps_done = ws->stats.steps_done;
  if (finite) *finite = ws->stats.finite;
  if (where == WEDG_HOST) {
    CK(ws, cudaMemcpy(u, ws->d_u, bU, cudaMemcpyDeviceToHost));
    CK(ws, cudaMemcpy(v, ws->d_v, bV, cudaMemcpyDeviceToHost));
  }
  return rc;
}

int wedg_batch_create(int n, wedg_ws *const *instances, wedg_batch **out) {
  if (!out) return WEDG_ERR_ARGUMENT;
  *out = nullptr;
  if (n < 1 || !instances) return WEDG_ERR_ARGUMENT;
  for (int i = 0; i < n; ++i)
    if (!instances[i]) return WEDG_ERR_ARGUMENT;
  wedg_batch *b = new wedg_batch();
  b->ws.assign(instances, instances + n);
  const size_t per = (size_t)2 * WEDG_BATCH_CHUNK * 4 * 8;    // doubles of one instance's table
  bool ok = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->half_done[0], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->half_done[1], cudaEventDisableTiming) == cudaSuccess &&
            cudaMallocHost(&b->h_tf, sizeof(double) * per * n) == cudaSuccess;
  for (int i = 0; i < n && ok; ++i) {
    cudaEvent_t e = nullptr;
    double *d = nullptr;
    ok = cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (ok) b->join.push_back(e);
    ok = ok && cudaMalloc(&d, sizeof(double) * per) == cudaSuccess;
    if (ok) b->d_tf.push_back(d);
  }
  if (!ok) {
    cudaGetLastError();
    delete b;
    return WEDG_ERR_CUDA;
  }
  *out = b;
  return WEDG_OK;
}

void wedg_batch_destroy(wedg_batch *b) { delete b; }

int wedg_batch_rk4_steps(wedg_batch *b, double *const *u_dev, double *const *v_dev, const double *t0,
                         const double *dt, int64_t nsteps, int stop_nonfinite, int64_t *steps_done, int *finite,
                         int *status) {
  if (!b || !u_dev || !v_dev || !t0 || !dt || nsteps < 0) return WEDG_ERR_ARGUMENT;
  const int n = (int)b->ws.size();
  const int64_t C = WEDG_BATCH_CHUNK;
  for (int i = 0; i < n; ++i)
    if (!u_dev[i] || !v_dev[i]) return WEDG_ERR_ARGUMENT;
  auto cuda_err = [&](cudaError_t e) {
    for (wedg_ws *w : b->ws) cuda_fail(w, e, "wedg_batch_rk4_steps");
    return WEDG_ERR_CUDA;
  };
#define BK(call)                                  \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_err(e_);   \
  } while (0)
  // ---- flags of every instance reset on its stream, before anything of the batch's stream
  for (int i = 0; i < n; ++i) {
    wedg_ws *w = b->ws[i];
    w->stats.kernel_launches = 0;
    int rc = reset_flags(w);
    if (rc) return rc;
    BK(cudaEventRecord(b->join[i], w->stream));
    BK(cudaStreamWaitEvent(b->main, b->join[i], 0));
  }
  // ---- the graph of one step of every instance, captured again when its key changed
  bool same = b->exec && b->gstop == (stop_nonfinite ? 1 : 0);
  for (int i = 0; i < n && same; ++i)
    same = b->gu[i] == u_dev[i] && b->gv[i] == v_dev[i] && b->gdt[i] == dt[i] && b->gshape[i] == b->ws[i]->shape_gen;
  if (!same) {
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    BK(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaEventRecord(b->fork, b->main);
    int rc = WEDG_OK;
    for (int i = 0; i < n && ce == cudaSuccess && rc == WEDG_OK; ++i) {
      wedg_ws *w = b->ws[i];
      ce = cudaStreamWaitEvent(w->stream, b->fork, 0);
      if (ce != cudaSuccess) break;
      const bool timing = w->timing;
      w->timing = false;
      rc = enqueue_rk4(w, u_dev[i], v_dev[i], 0.0, dt[i], stop_nonfinite ? 1 : 0, b->d_tf[i], 2 * C);
      w->timing = timing;
      if (rc == WEDG_OK) ce = cudaEventRecord(b->join[i], w->stream);
      if (ce == cudaSuccess && rc == WEDG_OK) ce = cudaStreamWaitEvent(b->main, b->join[i], 0);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ce2 = cudaStreamEndCapture(b->main, &g);
    if (rc != WEDG_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess || ce2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return cuda_err(ce != cudaSuccess ? ce : ce2);
    }
    b->graph = g;
    BK(cudaGraphInstantiate(&b->exec, g, 0));
    b->gu.assign(u_dev, u_dev + n);
    b->gv.assign(v_dev, v_dev + n);
    b->gdt.assign(dt, dt + n);
    b->gshape.resize(n);
    for (int i = 0; i < n; ++i) b->gshape[i] = b->ws[i]->shape_gen;
    b->gstop = stop_nonfinite ? 1 : 0;
  }
  // ---- the steps, one chunk of factor tables at a time (double-buffered, host and device)
  const size_t chunk = (size_t)C * 4 * 8;
  std::vector<double> t(t0, t0 + n);
  for (int64_t c = 0; c * C < nsteps; ++c) {
    const int half = (int)(c & 1);
    const int64_t cnt = std::min<int64_t>(C, nsteps - c * C);
    if (c >= 2) BK(cudaEventSynchronize(b->half_done[half]));   // its last upload has been read
    double *h = b->h_tf + (size_t)half * n * chunk;
    for (int i = 0; i < n; ++i) {
      factor_table(b->ws[i], t[i], dt[i], cnt, h + (size_t)i * chunk);
      for (int64_t it = 0; it < cnt; ++it) t[i] += dt[i];
    }
    for (int i = 0; i < n; ++i)
      BK(cudaMemcpyAsync(b->d_tf[i] + (size_t)half * chunk, h + (size_t)i * chunk, sizeof(double) * cnt * 32,
                         cudaMemcpyHostToDevice, b->main));
    BK(cudaEventRecord(b->half_done[half], b->main));
    for (int64_t it = 0; it < cnt; ++it) BK(cudaGraphLaunch(b->exec, b->main));
  }
  BK(cudaStreamSynchronize(b->main));
#undef BK
  int first = WEDG_OK;
  for (int i = 0; i < n; ++i) {
    wedg_ws *w = b->ws[i];
    w->stats.kernel_launches = 0;
    const int rc = collect(w);
    if (steps_done) steps_done[i] = w->stats.steps_done;
    if (finite) finite[i] = w->stats.finite;
    if (status) status[i] = rc;
    if (rc != WEDG_OK && first == WEDG_OK) first = rc;
  }
  return first;
}

int wedg_batch_autotune(wedg_batch *b, double *const *u_dev, double *const *v_dev, const double *t0,
                        const double *dt, int64_t steps, double *best_ms) {
  if (!b || !u_dev || !v_dev || !t0 || !dt || steps < 1) return WEDG_ERR_ARGUMENT;
  const int n = (int)b->ws.size();
  std::vector<double *> su(n), sv(n);
  std::vector<double> t1(n);
  for (int i = 0; i < n; ++i) {
    if (!u_dev[i] || !v_dev[i]) return WEDG_ERR_ARGUMENT;
    su[i] = b->ws[i]->d_u;
    sv[i] = b->ws[i]->d_v;
    t1[i] = t0[i] + dt[i];
  }
  // buckets of instances with the same degrees (the same kernels)
  std::vector<std::pair<int, int>> keys;
  std::vector<std::vector<int>> bucket;
  for (int i = 0; i < n; ++i) {
    const std::pair<int, int> key(b->ws[i]->nu, b->ws[i]->nv);
    size_t k = 0;
    while (k < keys.size() && keys[k] != key) ++k;
    if (k == keys.size()) { keys.push_back(key); bucket.emplace_back(); }
    bucket[k].push_back(i);
  }
  // steps steps of the batch from copies of the states, after one untimed step (which captures
  // the graph), with the present shapes
  auto trial = [&](double &ms) -> int {
    for (int i = 0; i < n; ++i) {
      wedg_ws *w = b->ws[i];
      const size_t bU = sizeof(double) * w->E * w->nu * w->nu, bV = sizeof(double) * w->E * w->nv * w->nv;
      cudaError_t e = cudaMemcpyAsync(su[i], u_dev[i], bU, cudaMemcpyDeviceToDevice, w->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(sv[i], v_dev[i], bV, cudaMemcpyDeviceToDevice, w->stream);
      if (e != cudaSuccess) return cuda_fail(w, e, "wedg_batch_autotune");
    }
    int rc = wedg_batch_rk4_steps(b, su.data(), sv.data(), t0, dt, 1, 0, nullptr, nullptr, nullptr);
    if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
    const auto c0 = std::chrono::steady_clock::now();
    rc = wedg_batch_rk4_steps(b, su.data(), sv.data(), t1.data(), dt, steps, 0, nullptr, nullptr, nullptr);
    ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - c0).count();
    return (rc == WEDG_WARN_CG_NOT_CONVERGED) ? WEDG_OK : rc;
  };
  double best = 0;
  int rc = trial(best);
  for (size_t k = 0; k < keys.size() && rc == WEDG_OK; ++k) {
    const std::vector<int> &ids = bucket[k];
    int bp = b->ws[ids[0]]->prep_threads, bm = b->ws[ids[0]]->mass_threads;
    for (int c = 0; c < 2 && rc == WEDG_OK; ++c)
      for (int q = 0; q < 3 && rc == WEDG_OK; ++q) {
        const int p = c == 0 ? kTuneThreads[q] : bp, m = c == 0 ? bm : kTuneThreads[q];
        if (p == bp && m == bm) continue;
        for (int i : ids) wedg_set_launch_shape(b->ws[i], p, m);
        double ms = 0;
        rc = trial(ms);
        if (rc == WEDG_OK && ms < kTuneGain * best) { best = ms; bp = p; bm = m; }
      }
    for (int i : ids) wedg_set_launch_shape(b->ws[i], bp, bm);   // also after a failed trial
  }
  if (rc != WEDG_OK) return rc;
  if (best_ms) *best_ms = best / steps;
  return WEDG_OK;
}

int wedg_run_source(wedg_ws *ws, double *u, double *v, const int64_t u_shape[4], const int64_t v_shape[4],
                    int where, const wedg_source_run *run, int64_t *steps_done, int *finite) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stats.kernel_launches = 0;
  int rc = check_shapes(ws, u_shape, v_shape);
  if (rc) return rc;
  if (!u || !v || !run) return argument_error(ws, "null argument");
  const int N = ws->N, E = ws->E, nu = ws->nu, nv = ws->nv, nq = ws->nq;
  if (run->nsteps < 0 || run->record_every < 1) return argument_error(ws, "nsteps must be ≥ 0 and record_every ≥ 1");
  if (run->nrec < 0 || (run->nrec > 0 && (!run->rec_j || !run->rec_k || !run->rec_py || !run->rec_px)))
    return argument_error(ws, "invalid receivers");
  if (run->slice_j < 0 || run->slice_j >= N || !run->slice_py) return argument_error(ws, "invalid slice");
  if (run->nsnap < 0 || (run->nsnap > 0 && !run->snap_after)) return argument_error(ws, "invalid snapshots");
  if (!run->err_c2 || !run->err_beta) return argument_error(ws, "err_c2 and err_beta are needed");
  for (int i = 0; i < run->nrec; ++i)
    if (run->rec_j[i] < 0 || run->rec_j[i] >= N || run->rec_k[i] < 0 || run->rec_k[i] >= N)
      return argument_error(ws, "receiver outside the mesh");
  for (int i = 0; i < run->nsnap; ++i)
    if (run->snap_after[i] < 1 || run->snap_after[i] > run->nsteps || (i && run->snap_after[i] <= run->snap_after[i - 1]))
      return argument_error(ws, "snapshot steps must increase within 1..nsteps");
  const int64_t nsteps = run->nsteps, every = run->record_every;
  const int64_t nrecord = nsteps / every + (nsteps % every ? 1 : 0);
  if ((nsteps * run->nrec && !run->recv) || (nrecord && (!run->energy || !run->vmax || !run->ndmin || !run->slices)) ||
      (run->nsnap && !run->snaps))
    return argument_error(ws, "null output array");

  // ---- the basis and mesh factors of the diagnostics
  DiagBasis B{};
  B.N = N; B.E = E; B.nu = nu; B.nv = nv;
  const double h = 1.0 / N;
  B.two_h = 2.0 / h;
  B.hh4 = h * h / 4;
  for (int i = 0; i < nq; ++i) {
    B.w[i] = ws->bh.w[i];
    for (int d = 0; d < nu; ++d) { B.P[i][d] = ws->bh.P[i][d]; B.S[i][d] = ws->bh.S[i][d]; }
  }

  // ---- device buffers of the run
  RunBuffers R;
  R.st = ws->stream;
  const size_t M = (size_t)N * nq, nE = (size_t)E * nq * nq;
  const int nblk = (E + DIAG_THREADS - 1) / DIAG_THREADS;
  int *d_rec_e;
  double *d_py, *d_px, *d_spy, *d_recv, *d_rec3, *d_part, *d_slices, *d_snaps, *d_c2, *d_be;
  CK(ws, R.get(&d_rec_e, run->nrec));
  CK(ws, R.get(&d_py, (size_t)run->nrec * nv));
  CK(ws, R.get(&d_px, (size_t)run->nrec * nv));
  CK(ws, R.get(&d_spy, nv));
  CK(ws, R.get(&d_recv, (size_t)nsteps * run->nrec));
  CK(ws, R.get(&d_rec3, 3 * (size_t)nrecord));
  CK(ws, R.get(&d_part, 3 * (size_t)nblk));
  CK(ws, R.get(&d_slices, (size_t)nrecord * M));
  CK(ws, R.get(&d_snaps, (size_t)run->nsnap * M * M));
  CK(ws, R.get(&d_c2, nE));
  CK(ws, R.get(&d_be, nE));
  std::vector<int> rec_e(run->nrec);
  for (int i = 0; i < run->nrec; ++i) rec_e[i] = run->rec_j[i] + N * run->rec_k[i];
  CK(ws, cudaMemcpyAsync(d_rec_e, rec_e.data(), sizeof(int) * run->nrec, cudaMemcpyHostToDevice, ws->stream));
  CK(ws, cudaMemcpyAsync(d_py, run->rec_py, sizeof(double) * run->nrec * nv, cudaMemcpyHostToDevice, ws->stream));
  CK(ws, cudaMemcpyAsync(d_px, run->rec_px, sizeof(double) * run->nrec * nv, cudaMemcpyHostToDevice, ws->stream));
  CK(ws, cudaMemcpyAsync(d_spy, run->slice_py, sizeof(double) * nv, cudaMemcpyHostToDevice, ws->stream));
  CK(ws, cudaMemcpyAsync(d_c2, run->err_c2, sizeof(double) * nE, cudaMemcpyHostToDevice, ws->stream));
  CK(ws, cudaMemcpyAsync(d_be, run->err_beta, sizeof(double) * nE, cudaMemcpyHostToDevice, ws->stream));

  // ---- the state
  const size_t bU = sizeof(double) * ws->E * nu * nu, bV = sizeof(double) * ws->E * nv * nv;
  double *du = u, *dv = v;
  if (where == WEDG_HOST) {
    CK(ws, cudaMemcpyAsync(ws->d_u, u, bU, cudaMemcpyHostToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(ws->d_v, v, bV, cudaMemcpyHostToDevice, ws->stream));
    du = ws->d_u; dv = ws->d_v;
  }
  if ((rc = reset_flags(ws))) return rc;

  // ---- the loop (src/solver.jl:933-952), all on the workspace stream
  double t = run->t0;
  int64_t ir = 0;
  int is = 0;
  const int tb = 128;
  for (int64_t it = 1; it <= nsteps; ++it) {
    if ((rc = enqueue_rk4(ws, du, dv, t, run->dt, 1))) return rc;
    t += run->dt;
    if (run->nrec) {
      k_receivers<<<(run->nrec + tb - 1) / tb, tb, 0, ws->stream>>>(dv, E, nv, run->nrec, d_rec_e, d_py, d_px,
                                                                   d_recv + (size_t)(it - 1) * run->nrec);
      ws->stats.kernel_launches += 1;
    }
    if (it % every == 0 || it == nsteps) {
      k_energy_elems<<<nblk, DIAG_THREADS, 0, ws->stream>>>(du, dv, B, d_c2, d_be, d_part);
      k_energy_final<<<1, DIAG_THREADS, 0, ws->stream>>>(d_part, nblk, d_rec3 + ir, d_rec3 + nrecord + ir,
                                                         d_rec3 + 2 * nrecord + ir);
      k_slice<<<(int)((M + tb - 1) / tb), tb, 0, ws->stream>>>(dv, B, run->slice_j, d_spy, d_slices + ir * M);
      ws->stats.kernel_launches += 3;
      ++ir;
    }
    if (is < run->nsnap && run->snap_after[is] == it) {
      k_vgrid<<<(unsigned)((M * M + tb - 1) / tb), tb, 0, ws->stream>>>(dv, B, d_snaps + (size_t)is * M * M);
      ws->stats.kernel_launches += 1;
      ++is;
    }
    CK(ws, cudaGetLastError());
  }
  rc = collect(ws);
  if (steps_done) *steps_done = ws->stats.steps_done;
  if (finite) *finite = ws->stats.finite;
  CK(ws, cudaMemcpy(run->recv, d_recv, sizeof(double) * nsteps * run->nrec, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(run->energy, d_rec3, sizeof(double) * nrecord, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(run->vmax, d_rec3 + nrecord, sizeof(double) * nrecord, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(run->ndmin, d_rec3 + 2 * nrecord, sizeof(double) * nrecord, cudaMemcpyDeviceToHost));
  CK(ws, cudaMemcpy(run->slices, d_slices, sizeof(double) * nrecord * M, cudaMemcpyDeviceToHost));
  if (run->nsnap) CK(ws, cudaMemcpy(run->snaps, d_snaps, sizeof(double) * run->nsnap * M * M, cudaMemcpyDeviceToHost));
  if (where == WEDG_HOST) {
    CK(ws, cudaMemcpy(u, ws->d_u, bU, cudaMemcpyDeviceToHost));
    CK(ws, cudaMemcpy(v, ws->d_v, bV, cudaMemcpyDeviceToHost));
  }
  return rc;
}

int wedg_rhs_adjoint(wedg_ws *ws, const double *u, const double *v, double t, const double *lam_u,
                     const double *lam_v, double *gu, double *gv, const int64_t u_shape[4], const int64_t v_shape[4],
                     int where) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stats.kernel_launches = 0;
  int rc = check_shapes(ws, u_shape, v_shape);
  if (rc) return rc;
  if (!u || !v || !lam_u || !lam_v || !gu || !gv) return argument_error(ws, "null pointer");
  if ((rc = adjoint_buffers(ws))) return rc;
  const size_t bU = sizeof(double) * ws->E * ws->nu * ws->nu, bV = sizeof(double) * ws->E * ws->nv * ws->nv;
  const double *du = u, *dv = v, *dlu = lam_u, *dlv = lam_v;
  double *dgu = gu, *dgv = gv;
  if (where == WEDG_HOST) {
    CK(ws, cudaMemcpyAsync(ws->adj_in[0], u, bU, cudaMemcpyHostToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(ws->adj_in[1], v, bV, cudaMemcpyHostToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(ws->adj_in[2], lam_u, bU, cudaMemcpyHostToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(ws->adj_in[3], lam_v, bV, cudaMemcpyHostToDevice, ws->stream));
    du = ws->adj_in[0]; dv = ws->adj_in[1]; dlu = ws->adj_in[2]; dlv = ws->adj_in[3];
    dgu = ws->d_ut; dgv = ws->d_vt;
  }
  if ((rc = reset_flags(ws))) return rc;
  if ((rc = enqueue_rhs_adjoint(ws, du, dv, t, dlu, dlv, dgu, dgv))) return rc;
  rc = collect(ws);
  if (where == WEDG_HOST) {
    CK(ws, cudaMemcpy(gu, ws->d_ut, bU, cudaMemcpyDeviceToHost));
    CK(ws, cudaMemcpy(gv, ws->d_vt, bV, cudaMemcpyDeviceToHost));
  }
  return rc;
}

int wedg_rk4_adjoint_forward(wedg_ws *ws, const double *u0, const double *v0, double t0, double dt, int64_t nsteps,
                             int64_t every, double *uT, double *vT, const int64_t u_shape[4],
                             const int64_t v_shape[4], int where) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stats.kernel_launches = 0;
  ws->rk_ready = false;
  int rc = check_shapes(ws, u_shape, v_shape);
  if (rc) return rc;
  if (!u0 || !v0) return argument_error(ws, "null pointer");
  if (nsteps < 0 || every < 1) return argument_error(ws, "nsteps must be ≥ 0 and the checkpoint interval ≥ 1");
  if ((rc = adjoint_buffers(ws))) return rc;
  const size_t nU = (size_t)ws->E * ws->nu * ws->nu, nV = (size_t)ws->E * ws->nv * ws->nv, n = nU + nV;
  const int64_t nchk = nsteps ? (nsteps + every - 1) / every : 0;
  const int64_t seg = std::min<int64_t>(every, std::max<int64_t>(nsteps, 1));
  // buffers: a state is u followed by v (n doubles)
  if (!ws->rk_lam) {
    if ((rc = dalloc(ws, &ws->rk_lam, n)) || (rc = dalloc(ws, &ws->rk_acc, n)) || (rc = dalloc(ws, &ws->rk_kbar, n)) ||
        (rc = dalloc(ws, &ws->rk_g, n)) || (rc = dalloc(ws, &ws->rk_y, n)) ||
        (rc = dalloc(ws, &ws->rk_par, 3 * (size_t)ws->E)))
      return rc;
  }
  while (ws->rk_chk_n < nchk) {
    double *p;
    if ((rc = dalloc(ws, &p, n))) return rc;
    ws->rk_chk.push_back(p);
    ++ws->rk_chk_n;
  }
  while (ws->rk_seg_n < 4 * seg) {
    double *p;
    if ((rc = dalloc(ws, &p, n))) return rc;
    ws->rk_seg.push_back(p);
    ++ws->rk_seg_n;
  }
  cudaStream_t st = ws->stream;
  const cudaMemcpyKind in = where == WEDG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  double *yu = ws->rk_y, *yv = ws->rk_y + nU;
  CK(ws, cudaMemcpyAsync(yu, u0, sizeof(double) * nU, in, st));
  CK(ws, cudaMemcpyAsync(yv, v0, sizeof(double) * nV, in, st));
  ws->rk_t.assign(nsteps + 1, t0);
  for (int64_t k = 0; k < nsteps; ++k) ws->rk_t[k + 1] = ws->rk_t[k] + dt;
  if ((rc = reset_flags(ws))) return rc;
  for (int64_t k = 0; k < nsteps; ++k) {
    if (k % every == 0) CK(ws, cudaMemcpyAsync(ws->rk_chk[k / every], ws->rk_y, sizeof(double) * n,
                                               cudaMemcpyDeviceToDevice, st));
    if ((rc = enqueue_rk4(ws, yu, yv, ws->rk_t[k], dt, 1))) return rc;
  }
  CK(ws, cudaGetLastError());
  rc = collect(ws);
  if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
  if (!ws->stats.finite) return argument_error(ws, "the forward run is not finite");
  const cudaMemcpyKind out = where == WEDG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (uT) CK(ws, cudaMemcpy(uT, yu, sizeof(double) * nU, out));
  if (vT) CK(ws, cudaMemcpy(vT, yv, sizeof(double) * nV, out));
  ws->rk_dt = dt;
  ws->rk_nsteps = nsteps;
  ws->rk_every = every;
  ws->rk_ready = true;
  return rc;
}

int wedg_rk4_adjoint_reverse(wedg_ws *ws, const double *lam_u, const double *lam_v, double *gu, double *gv,
                             double *g_c2, double *g_alpha, double *g_beta, int where) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stats.kernel_launches = 0;
  if (!ws->rk_ready) return argument_error(ws, "no forward run with checkpoints (wedg_rk4_adjoint_forward) to reverse");
  if (!lam_u || !lam_v || !gu || !gv) return argument_error(ws, "null pointer");
  const bool params = g_c2 || g_alpha || g_beta;
  if (params && !(g_c2 && g_alpha && g_beta)) return argument_error(ws, "give all three parameter gradients or none");
  if (params && (!ws->fast || !ws->cfg.src_on || ws->cfg.mms_on))
    return argument_error(ws, "parameter gradients need source mode and c², α, β constant on each element");
  int rc;
  const size_t nU = (size_t)ws->E * ws->nu * ws->nu, nV = (size_t)ws->E * ws->nv * ws->nv, n = nU + nV;
  const int64_t nsteps = ws->rk_nsteps, every = ws->rk_every;
  const int64_t nchk = nsteps ? (nsteps + every - 1) / every : 0;
  const double dt = ws->rk_dt;
  const std::vector<double> &t = ws->rk_t;
  cudaStream_t st = ws->stream;
  double *yu = ws->rk_y, *yv = ws->rk_y + nU;
  const cudaMemcpyKind in = where == WEDG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  CK(ws, cudaMemcpyAsync(ws->rk_lam, lam_u, sizeof(double) * nU, in, st));
  CK(ws, cudaMemcpyAsync(ws->rk_lam + nU, lam_v, sizeof(double) * nV, in, st));
  if (params) CK(ws, cudaMemsetAsync(ws->rk_par, 0, sizeof(double) * 3 * ws->E, st));
  if ((rc = reset_flags(ws))) return rc;
  const int lb = 256, lg = (int)std::min<size_t>((n + lb - 1) / lb, 152 * 16);
  auto lin = [&](double *out, double a, const double *x, double b, const double *y, const double *z) {
    k_lincomb<<<lg, lb, 0, st>>>(n, out, a, x, b, y, z);
    ws->stats.kernel_launches += 1;
  };
  // keep the forward data of every stage of a segment when it fits the memory allowance
  const int64_t seg = std::min<int64_t>(every, std::max<int64_t>(nsteps, 1));
  const size_t keep_bytes = (size_t)(4 * seg) * stage_data_bytes(ws);
  size_t have = 0;
  for (size_t i = 0; i < ws->rk_keep.size(); ++i) have += stage_data_bytes(ws);
  bool keep = false;
  if (ws->adj_mem < 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) keep = keep_bytes <= (fr + have) / 2;
  } else {
    keep = keep_bytes <= (size_t)ws->adj_mem;
  }
  if (keep) {
    const size_t E = ws->E;
    const size_t nd = (size_t)ws->nu * ws->nu + ws->nv * ws->nv + 12 * ws->nq + ws->qh * ws->qh + 2;
    while ((int64_t)ws->rk_keep.size() < 4 * seg) {
      wedg_ws::StageData d;
      double *b;
      int *ib;
      if ((rc = dalloc(ws, &b, nd * E)) || (rc = dalloc(ws, &ib, E * (1 + NBIN) + 2 * NBIN))) return rc;
      d.k = b;
      d.tr = d.k + n;
      d.G = d.tr + 12 * (size_t)ws->nq * E;
      d.th = d.G + (size_t)ws->qh * ws->qh * E;
      d.de = d.th + E;
      d.nst = ib;
      d.bins = ib + E;
      d.bin_count = ib + E * (1 + NBIN);
      ws->rk_keep.push_back(d);
    }
  }
  // ---- reverse pass, segment by segment
  for (int64_t c = nchk - 1; c >= 0; --c) {
    const int64_t k0 = c * every, k1 = std::min(nsteps, k0 + every);
    CK(ws, cudaMemcpyAsync(ws->rk_y, ws->rk_chk[c], sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    for (int64_t k = k0; k < k1; ++k) {
      if (keep) {
        // the step as four RHS evaluations (their outputs and data kept) and the RK4 combinations:
        // Y1 = y, Y_{s+1} = y + c_s K_s, y ← y + dt/6 (K1 + 2K2 + 2K3 + K4)
        const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
        const double ts[4] = {t[k], t[k] + 0.5 * dt, t[k] + 0.5 * dt, t[k] + dt};
        CK(ws, cudaMemcpyAsync(ws->rk_seg[4 * (k - k0)], ws->rk_y, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        for (int s = 0; s < 4; ++s) {
          wedg_ws::StageData &d = ws->rk_keep[4 * (k - k0) + s];
          const double *Y = ws->rk_seg[4 * (k - k0) + s];
          StageIO S{};
          S.xu = Y; S.xv = Y + nU;
          stage_factors(ws, ts[s], S);
          S.mode = OUT_RHS;
          S.ut = d.k;
          S.vt = d.k + nU;
          CK(ws, cudaMemsetAsync(d.bin_count, 0, 2 * NBIN * sizeof(int), st));
          d.parity = ws->parity;
          const Fields Fk = kept_fields(ws, d);
          if ((rc = enqueue_stage(ws, S, &Fk))) return rc;
          if (s < 3) lin(ws->rk_seg[4 * (k - k0) + s + 1], cs[s], d.k, 1.0, ws->rk_y, nullptr);
        }
        const double *K[4] = {ws->rk_keep[4 * (k - k0)].k, ws->rk_keep[4 * (k - k0) + 1].k,
                              ws->rk_keep[4 * (k - k0) + 2].k, ws->rk_keep[4 * (k - k0) + 3].k};
        lin(ws->rk_acc, 2.0, K[1], 1.0, K[0], nullptr);
        lin(ws->rk_acc, 2.0, K[2], 1.0, K[3], ws->rk_acc);
        lin(ws->rk_y, dt / 6.0, ws->rk_acc, 1.0, ws->rk_y, nullptr);
        continue;
      }
      double *su[4], *sv[4];
      for (int s = 0; s < 4; ++s) {
        su[s] = ws->rk_seg[4 * (k - k0) + s];
        sv[s] = su[s] + nU;
      }
      if ((rc = enqueue_rk4(ws, yu, yv, t[k], dt, 1, nullptr, 0, su, sv))) return rc;
    }
    for (int64_t k = k1 - 1; k >= k0; --k) {
      const double ts[4] = {t[k], t[k] + 0.5 * dt, t[k] + 0.5 * dt, t[k] + dt};
      // K̄_s = ca[s] λ + cb[s] Ȳ_{s+1}, Ȳ = Jᵀ K̄ at the stage state: y_{n+1} = y + dt/6 (K1 + 2K2 +
      // 2K3 + K4), Y2 = y + dt/2 K1, Y3 = y + dt/2 K2, Y4 = y + dt K3
      const double ca[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};
      const double cb[4] = {0.5 * dt, 0.5 * dt, dt, 0.0};
      for (int s = 3; s >= 0; --s) {
        lin(ws->rk_kbar, ca[s], ws->rk_lam, cb[s], s == 3 ? nullptr : ws->rk_g, nullptr);
        const double *Y = ws->rk_seg[4 * (k - k0) + s];
        double *gpar = params ? ws->rk_par : nullptr;
        if (keep) {
          const wedg_ws::StageData &d = ws->rk_keep[4 * (k - k0) + s];
          StageIO S{};
          S.xu = Y; S.xv = Y + nU;
          stage_factors(ws, ts[s], S);
          S.parity = d.parity;
          S.ut = d.k;
          S.vt = d.k + nU;
          rc = enqueue_adjoint_core(ws, kept_fields(ws, d), S, ws->rk_kbar, ws->rk_kbar + nU, ws->rk_g,
                                    ws->rk_g + nU, gpar);
        } else {
          rc = enqueue_rhs_adjoint(ws, Y, Y + nU, ts[s], ws->rk_kbar, ws->rk_kbar + nU, ws->rk_g, ws->rk_g + nU,
                                   gpar);
        }
        if (rc) return rc;
        lin(ws->rk_acc, 1.0, s == 3 ? ws->rk_lam : ws->rk_acc, 1.0, ws->rk_g, nullptr);
      }
      std::swap(ws->rk_lam, ws->rk_acc);
    }
  }
  CK(ws, cudaGetLastError());
  rc = collect(ws);
  const cudaMemcpyKind out = where == WEDG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  CK(ws, cudaMemcpy(gu, ws->rk_lam, sizeof(double) * nU, out));
  CK(ws, cudaMemcpy(gv, ws->rk_lam + nU, sizeof(double) * nV, out));
  if (params) {
    CK(ws, cudaMemcpy(g_c2, ws->rk_par, sizeof(double) * ws->E, out));
    CK(ws, cudaMemcpy(g_alpha, ws->rk_par + ws->E, sizeof(double) * ws->E, out));
    CK(ws, cudaMemcpy(g_beta, ws->rk_par + 2 * ws->E, sizeof(double) * ws->E, out));
  }
  return rc;
}

int wedg_set_launch_shape(wedg_ws *ws, int prep_threads, int mass_threads) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  auto ok = [](int t) { return t >= 32 && t <= CHEB_THREADS && t % 32 == 0; };
  if (!ok(prep_threads) || !ok(mass_threads))
    return argument_error(ws, "launch shapes are 32, 64, 96 or 128 threads per block");
  if (prep_threads != ws->prep_threads || mass_threads != ws->mass_threads) {
    ws->prep_threads = prep_threads;
    ws->mass_threads = mass_threads;
    ++ws->shape_gen;
  }
  return WEDG_OK;
}

int wedg_get_launch_shape(const wedg_ws *ws, int *prep_threads, int *mass_threads) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  if (prep_threads) *prep_threads = ws->prep_threads;
  if (mass_threads) *mass_threads = ws->mass_threads;
  return WEDG_OK;
}

int wedg_autotune(wedg_ws *ws, const double *u_dev, const double *v_dev, double t0, double dt, int64_t steps,
                  double *best_ms) {
  if (!ws || !u_dev || !v_dev || steps < 1) return WEDG_ERR_ARGUMENT;
  const size_t bU = sizeof(double) * ws->E * ws->nu * ws->nu, bV = sizeof(double) * ws->E * ws->nv * ws->nv;
  cudaEvent_t e0 = take_event(ws), e1 = take_event(ws);
  // steps RK4 steps from copies of the state (in the workspace's own state buffers), after one
  // untimed step, with the shapes (p, m)
  auto trial = [&](int p, int m, double &ms) -> int {
    int rc = wedg_set_launch_shape(ws, p, m);
    if (rc) return rc;
    CK(ws, cudaMemcpyAsync(ws->d_u, u_dev, bU, cudaMemcpyDeviceToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(ws->d_v, v_dev, bV, cudaMemcpyDeviceToDevice, ws->stream));
    if ((rc = reset_flags(ws)) || (rc = enqueue_rk4(ws, ws->d_u, ws->d_v, t0, dt, 0))) return rc;
    CK(ws, cudaEventRecord(e0, ws->stream));
    double t = t0 + dt;
    for (int64_t it = 0; it < steps; ++it, t += dt)
      if ((rc = enqueue_rk4(ws, ws->d_u, ws->d_v, t, dt, 0))) return rc;
    CK(ws, cudaEventRecord(e1, ws->stream));
    CK(ws, cudaStreamSynchronize(ws->stream));
    rc = collect(ws);
    if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
    float f = 0;
    CK(ws, cudaEventElapsedTime(&f, e0, e1));
    ms = f;
    return WEDG_OK;
  };
  int bp = ws->prep_threads, bm = ws->mass_threads;
  double best = 0;
  int rc = trial(bp, bm, best);
  for (int c = 0; c < 2 && rc == WEDG_OK; ++c)
    for (int k = 0; k < 3 && rc == WEDG_OK; ++k) {
      const int p = c == 0 ? kTuneThreads[k] : bp, m = c == 0 ? bm : kTuneThreads[k];
      if (p == bp && m == bm) continue;
      double ms = 0;
      rc = trial(p, m, ms);
      if (rc == WEDG_OK && ms < kTuneGain * best) { best = ms; bp = p; bm = m; }
    }
  ws->ev_pool.push_back(e0);
  ws->ev_pool.push_back(e1);
  wedg_set_launch_shape(ws, bp, bm);            // the best shape so far, also after a failed trial
  if (rc != WEDG_OK) return rc;
  if (best_ms) *best_ms = best / steps;
  return WEDG_OK;
}

int wedg_set_adjoint_memory(wedg_ws *ws, int64_t bytes) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->adj_mem = bytes < 0 ? -1 : bytes;
  return WEDG_OK;
}

int wedg_rk4_adjoint(wedg_ws *ws, const double *u0, const double *v0, double t0, double dt, int64_t nsteps,
                     int64_t every, const double *lam_u, const double *lam_v, double *gu, double *gv,
                     double *g_c2, double *g_alpha, double *g_beta, const int64_t u_shape[4],
                     const int64_t v_shape[4], int where) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  if (!lam_u || !lam_v || !gu || !gv) return argument_error(ws, "null pointer");
  int rc = wedg_rk4_adjoint_forward(ws, u0, v0, t0, dt, nsteps, every, nullptr, nullptr, u_shape, v_shape, where);
  if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
  return wedg_rk4_adjoint_reverse(ws, lam_u, lam_v, gu, gv, g_c2, g_alpha, g_beta, where);
}

int wedg_rk4_step(wedg_ws *ws, double *u, double *v, double t, double dt, const int64_t u_shape[4],
                  const int64_t v_shape[4], int where, int *finite) {
  return wedg_rk4_steps(ws, u, v, t, dt, 1, u_shape, v_shape, where, 0, nullptr, finite);
}

int wedg_rk4_steps_async(wedg_ws *ws, double *u_dev, double *v_dev, double t0, double dt, int64_t nsteps) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stats.kernel_launches = 0;
  int rc = reset_flags(ws);
  if (rc) return rc;
  double t = t0;
  for (int64_t it = 0; it < nsteps; ++it) {
    if ((rc = enqueue_rk4(ws, u_dev, v_dev, t, dt, 0))) return rc;
    t += dt;
  }
  return WEDG_OK;
}

int wedg_sync_status(wedg_ws *ws, int64_t *steps_done, int *finite) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  int rc = collect(ws);
  if (steps_done) *steps_done = ws->stats.steps_done;
  if (finite) *finite = ws->stats.finite;
  return rc;
}

int wedg_error_message(const wedg_ws *ws, char *buf, size_t len) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  if (buf && len) {
    std::strncpy(buf, ws->message.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return ws->status;
}

int64_t wedg_error_key(const wedg_ws *ws) { return ws ? ws->key : 0; }

int wedg_get_stats(const wedg_ws *ws, wedg_stats *out) {
  if (!ws || !out) return WEDG_ERR_ARGUMENT;
  *out = ws->stats;
  return WEDG_OK;
}

void *wedg_get_stream(const wedg_ws *ws) { return ws ? (void *)ws->stream : nullptr; }

int wedg_set_stream(wedg_ws *ws, void *stream) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->stream = stream ? (cudaStream_t)stream : ws->own_stream;
  return WEDG_OK;
}

int wedg_time_kernels(wedg_ws *ws, int enable) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  ws->timing = enable != 0;
  return WEDG_OK;
}

int wedg_kernel_times(wedg_ws *ws, double *prep_ms, int64_t *prep_launches, double *stage_ms,
                      int64_t *stage_launches, double *mass_ms, int64_t *mass_launches, int reset) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  CK(ws, cudaStreamSynchronize(ws->stream));
  drain_events(ws);
  if (prep_ms) *prep_ms = ws->t_prep;
  if (prep_launches) *prep_launches = ws->n_prep;
  if (stage_ms) *stage_ms = ws->t_stage;
  if (stage_launches) *stage_launches = ws->n_stage;
  if (mass_ms) *mass_ms = ws->t_mass;
  if (mass_launches) *mass_launches = ws->n_mass;
  if (reset) { ws->t_prep = ws->t_stage = ws->t_mass = 0; ws->n_prep = ws->n_stage = ws->n_mass = 0; }
  return WEDG_OK;
}

const char *wedg_status_string(int status) {
  switch (status) {
    case WEDG_OK: return "ok";
    case WEDG_ERR_DIMENSION: return "dimension mismatch";
    case WEDG_ERR_BOUNDARY_WEIGHT: return "boundary weight not positive";
    case WEDG_ERR_MASS_NOT_PD: return "mass matrix not positive definite";
    case WEDG_WARN_CG_NOT_CONVERGED: return "CG did not reach the tolerance";
    case WEDG_ERR_TIMEOUT: return "device wait timed out";
    case WEDG_ERR_CUDA: return "CUDA error";
    case WEDG_ERR_ARGUMENT: return "invalid argument";
    case WEDG_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char *wedg_version(void) { return "libwedg 0.1 (sm_103a, FP64)"; }

}  // extern "C"
