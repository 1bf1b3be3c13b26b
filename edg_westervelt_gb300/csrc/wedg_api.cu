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

// k_lincomb for many instances in one launch (blockIdx.y is the instance): out = a x + b y (+ z)
struct LinPtrs {
  size_t n;
  double *out;
  const double *x, *y, *z;
};
constexpr int LIN_CAP = 64;
struct LinMulti {
  int n;
  double a, b;
  LinPtrs p[LIN_CAP];
};
__global__ void k_lincomb_m(const __grid_constant__ LinMulti L) {
  const LinPtrs &q = L.p[blockIdx.y];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < q.n; i += (size_t)gridDim.x * blockDim.x) {
    double r = L.a * q.x[i];
    if (q.y) r = fma(L.b, q.y[i], r);
    if (q.z) r += q.z[i];
    q.out[i] = r;
  }
}

// k_step_done for many instances in one launch (thread i: instance i), flags in the parameters
struct StepFlagsP {
  unsigned long long *err;
  const unsigned int *nonfinite;
  long long *steps_done;
};
struct StepMulti {
  int n, stop_nonfinite;
  StepFlagsP f[LIN_CAP];
};
__global__ void k_step_done_p(const __grid_constant__ StepMulti P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const StepFlagsP &x = P.f[i];
  if (*x.err != ERR_NONE) return;
  *x.steps_done += 1;
  if (P.stop_nonfinite && *x.nonfinite) *x.err = (3ull << ERR_CLASS_SHIFT);
}

// The candidates of the autotuners, tried one coordinate at a time (k_prep's block, then the
// mass solves'); a candidate replaces the best so far only when it is faster by more than 2 %
const int kTuneThreads[3] = {32, 64, 128};
constexpr double kTuneGain = 0.98;
constexpr int kTuneRepeats = 3;   // paired trials of the batch autotuner
// RK4 steps of the batch's larger graph: within it an instance starts its next step as soon as its
// own step is done (the table chunk, WEDG_BATCH_CHUNK steps, is a multiple of it)
constexpr int kBatchGraphSteps = 4;
// element ranges in which a host state is copied in while the first k_prep runs on the ranges that
// have arrived
constexpr int kCopyChunks = 4;
static_assert(WEDG_BATCH_CHUNK % kBatchGraphSteps == 0, "a table chunk holds whole multi-step graphs");

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

namespace {

// The flags of a workspace (or of every instance of a batch), reset and read back by one launch each
struct BatchFlagPtrs {
  unsigned long long *err, *nsum;
  unsigned int *cg_nfail, *nonfinite;
  int *nmax, *bin_count;
  long long *steps_done;
};
struct BatchFlagVals {
  unsigned long long err, nsum;
  long long done;
  unsigned int cgf, nonf;
  int nmax, pad;
};

// reset_flags of instance blockIdx.x
__global__ void k_batch_reset(const BatchFlagPtrs *p, int n) {
  if ((int)blockIdx.x >= n) return;
  const BatchFlagPtrs f = p[blockIdx.x];
  for (int t = threadIdx.x; t < 2 * NBIN; t += blockDim.x) f.bin_count[t] = 0;
  if (threadIdx.x == 0) {
    *f.err = ERR_NONE;
    *f.nsum = 0;
    *f.cg_nfail = 0;
    *f.nonfinite = 0;
    f.nmax[0] = f.nmax[1] = f.nmax[2] = 0;
    *f.steps_done = 0;
  }
}

// the flags collect reads, of every instance
__global__ void k_batch_read(const BatchFlagPtrs *p, int n, BatchFlagVals *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BatchFlagPtrs f = p[i];
  out[i] = BatchFlagVals{*f.err, *f.nsum, *f.steps_done, *f.cg_nfail, *f.nonfinite, f.nmax[2], 0};
}

}  // namespace

struct wedg_ws {
  wedg_config cfg;
  int N = 0, E = 0, nu = 0, nv = 0, nq = 0, qh = 0;
  bool fast = false;
  Launchers L;
  BasisHost bh;
  std::vector<char> basis;
  Fields F{};
  bool modal_ok = false;   // the traces may be kept as modal end sums (Fields::modal)
  // the flags' pointers and their values after a call (h_flagv pinned): one reset and one read
  BatchFlagPtrs *d_flagp = nullptr;
  BatchFlagVals *d_flagv = nullptr, *h_flagv = nullptr;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  // host-state calls: copies beside the workspace's stream (created on first use)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_copy[2] = {nullptr, nullptr};
  cudaEvent_t ev_chunk[kCopyChunks] = {};
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
  double *rk_ry = nullptr, *rk_racc = nullptr;   // the recompute's state and RK4 sum when it runs beside the reverse
  // the forward run the next reverse sweep differentiates
  bool rk_ready = false;
  double rk_dt = 0;
  int64_t rk_nsteps = 0, rk_every = 1;
  std::vector<double> rk_t;
  // the forward data of every stage of one segment, kept by the reverse sweep (see
  // wedg_set_adjoint_memory): the stage RHS K = (ut | vt), traces, G, Chebyshev data
  struct StageData {
    double *k = nullptr, *tr = nullptr, *G = nullptr, *th = nullptr, *de = nullptr;
    int *nst = nullptr, *bins = nullptr, *bin_count = nullptr, *nmax = nullptr;
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

// The point traces of the adjoint calls: the adjoint kernels read the traces at the face points,
// so the forward kernels these calls run keep point traces while the guard lives
struct PointTraces {
  std::vector<wedg_ws *> G;
  explicit PointTraces(const std::vector<wedg_ws *> &g) : G(g) {
    for (wedg_ws *w : G) w->F.modal = 0;
  }
  ~PointTraces() {
    for (wedg_ws *w : G) w->F.modal = w->modal_ok ? 1 : 0;
  }
};

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
  k_batch_reset<<<1, 128, 0, ws->stream>>>(ws->d_flagp, 1);
  CK(ws, cudaGetLastError());
  ws->parity = 0;
  ws->stats.element_stages = 0;
  return WEDG_OK;
}

// The copy stream and its two events of host-state calls (created on first use)
int copy_stream_ready(wedg_ws *ws) {
  if (ws->copy_stream) return WEDG_OK;
  CK(ws, cudaEventCreateWithFlags(&ws->ev_copy[0], cudaEventDisableTiming));
  CK(ws, cudaEventCreateWithFlags(&ws->ev_copy[1], cudaEventDisableTiming));
  for (cudaEvent_t &e : ws->ev_chunk) CK(ws, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CK(ws, cudaStreamCreateWithFlags(&ws->copy_stream, cudaStreamNonBlocking));
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

// enqueue the three kernels of one stage (on the workspace's Fields, or on Fo); after_stage, when
// given, is recorded on the stream after the stage kernel; with prep_done the stage's k_prep has
// been enqueued already (by ranges of elements, with this stage's bin parity)
int enqueue_stage(wedg_ws *ws, const StageIO &S, const Fields *Fo = nullptr, cudaEvent_t after_stage = nullptr,
                  bool prep_done = false) {
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
  if (!prep_done) CK(ws, ws->L.prep(ws->basis.data(), F, Sp, bp, tp, ws->stream, 0));
  if (ws->timing) cudaEventRecord(e1, ws->stream);
  CK(ws, ws->L.stage(ws->basis.data(), F, Sp, bs, ts, ws->stream));
  if (after_stage) CK(ws, cudaEventRecord(after_stage, ws->stream));
  if (ws->timing) cudaEventRecord(e2, ws->stream);
  CK(ws, ws->L.mass(ws->basis.data(), F, Sp, bm, ws->mass_threads, ws->stream));
  if (ws->timing) {
    cudaEventRecord(e3, ws->stream);
    ws->ev_pending.push_back({e0, e1, e2, e3});
  }
  ws->stats.kernel_launches += prep_done ? 2 : 3;
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

// The StageIO of stage s (0..3) of an RK4 step of the state (u, v) at time t (src/solver.jl:299-321):
// its input state, time factors (or, with tf, the device table of tf_n steps indexed by the
// workspace's step counter, for graph replays) and outputs. With stage_u, stage_v (four buffers
// each) the stage states Y1..Y4 are kept there.
StageIO rk4_stage_io(const wedg_ws *ws, double *u, double *v, int s, double t, double dt, const double *tf,
                     long long tf_n, double *const *stage_u, double *const *stage_v) {
  const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
  const double ts[4] = {t, t + 0.5 * dt, t + 0.5 * dt, t + dt};
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
    S.mode = ws->cfg.mass_solver == WEDG_CG ? OUT_RK4_LAST_ACC : OUT_RK4_LAST;
    S.c = dt / 6.0;
  }
  return S;
}

// One RK4 step on the workspace stream. With tf != nullptr the stage kernels take their time
// factors from the device table tf (tf_n steps, indexed by the device step counter), so that the
// launches can be captured once into a CUDA graph and replayed for every step. u_final, when
// given (Chebyshev mass solves only), is recorded once the last stage's k_stage has written the
// step's u: nothing of the step writes u after it.
int enqueue_rk4(wedg_ws *ws, double *u, double *v, double t, double dt, int stop_nonfinite,
                const double *tf = nullptr, long long tf_n = 0, double *const *stage_u = nullptr,
                double *const *stage_v = nullptr, cudaEvent_t u_final = nullptr, bool first_prep_done = false) {
  // with stage_u, stage_v (four buffers each) the stage states Y1..Y4 of the step are kept there
  const bool cg = ws->cfg.mass_solver == WEDG_CG;
  if (stage_u) {
    const size_t bU = sizeof(double) * ws->E * ws->nu * ws->nu, bV = sizeof(double) * ws->E * ws->nv * ws->nv;
    CK(ws, cudaMemcpyAsync(stage_u[0], u, bU, cudaMemcpyDeviceToDevice, ws->stream));
    CK(ws, cudaMemcpyAsync(stage_v[0], v, bV, cudaMemcpyDeviceToDevice, ws->stream));
  }
  for (int s = 0; s < 4; ++s) {
    int rc = enqueue_stage(ws, rk4_stage_io(ws, u, v, s, t, dt, tf, tf_n, stage_u, stage_v), nullptr,
                           s == 3 && !cg ? u_final : nullptr, s == 0 && first_prep_done);
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
  CK(ws, ws->L.mass(ws->basis.data(), Fm, Sm, 1, ws->mass_threads, ws->stream));
  // ν = A_e⁻¹ λ_u
  StageIO Su = S;
  Su.mode = OUT_ADJ_USOLVE;
  Su.xu = lam_u;
  Su.ut = ws->adj_nu;
  CK(ws, ws->L.stage(ws->basis.data(), Fs, Su, bs, ts, ws->stream));
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
  CK(ws, ws->L.stage(ws->basis.data(), Fs, Sv, bs, ts, ws->stream));
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
  F.nst = d.nst; F.bins = d.bins; F.bin_count = d.bin_count; F.nmax = d.nmax;
  return F;
}

// bytes of the kept data of one stage
size_t stage_data_bytes(const wedg_ws *ws) {
  const size_t E = ws->E;
  return sizeof(double) * E * ((size_t)ws->nu * ws->nu + ws->nv * ws->nv + 12 * ws->nq + ws->qh * ws->qh + 2) +
         sizeof(int) * (E * (1 + NBIN) + 2 * NBIN + 4);
}

// The status and statistics of a call from the workspace's flags (read back after the call)
int apply_flags(wedg_ws *ws, unsigned long long err, unsigned int cgf, unsigned int nonf, int nmax, long long done,
                unsigned long long nsum) {
  ws->stats.cheb_steps_sum = (int64_t)nsum;
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

int collect(wedg_ws *ws) {
  k_batch_read<<<1, 32, 0, ws->stream>>>(ws->d_flagp, 1, ws->d_flagv);
  CK(ws, cudaGetLastError());
  CK(ws, cudaMemcpyAsync(ws->h_flagv, ws->d_flagv, sizeof(BatchFlagVals), cudaMemcpyDeviceToHost, ws->stream));
  CK(ws, cudaStreamSynchronize(ws->stream));
  drain_events(ws);
  const BatchFlagVals &f = *ws->h_flagv;
  return apply_flags(ws, f.err, f.cgf, f.nonf, f.nmax, f.done, f.nsum);
}


int argument_error(wedg_ws *ws, const std::string &msg) {
  if (ws) {
    ws->status = WEDG_ERR_ARGUMENT;
    ws->message = msg;
  }
  return WEDG_ERR_ARGUMENT;
}

// ---- multi-instance launches of one kernel over many instances' arguments, in chunks of the
//      launch's capacity (wedg_kernels.cuh); kind 0: k_prep (tile = threads), 1: k_stage
//      (tile = stage_threads), 2: the mass solve (tile = teams of `threads`). grid_of maps the
//      virtual blocks of a chunk to its physical grid (persistent launches).
enum { MK_PREP = 0, MK_STAGE = 1, MK_MASS = 2 };
template <class GridOf>
cudaError_t multi_stage_launch(const Launchers &L, const void *basis, int nu, int nv, bool fast, int kind,
                               const std::vector<StageArgs> &args, int threads, cudaStream_t st, GridOf grid_of) {
  const int TPW = 32 / (qhigh(nu, nv) / 2 + (qhigh(nu, nv) & 1));
  const int tile = kind == MK_PREP ? threads : kind == MK_STAGE ? stage_threads(nu, nv, fast) : (threads / 32) * TPW;
  const int n = (int)args.size();
  for (int c0 = 0; c0 < n; c0 += MultiStage::cap) {
    const int m = std::min(n - c0, MultiStage::cap);
    MultiStage P;
    P.n = m;
    P.tile = tile;
    P.first[0] = 0;
    for (int x = 0; x < m; ++x) {
      P.a[x] = args[c0 + x];
      P.first[x + 1] = P.first[x] + (P.a[x].F.E + tile - 1) / tile;
    }
    const int grid = grid_of(kind, P.first[m]);
    const cudaError_t e = kind == MK_PREP    ? L.prep_m(basis, P, grid, threads, st)
                          : kind == MK_STAGE ? L.stage_m(basis, P, grid, stage_threads(nu, nv, fast), st)
                                             : L.mass_m(basis, P, grid, threads, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// kind 0: k_adj_hats, 1: k_adj_mass, 2: k_adj_face (one virtual block per tile, no persistence)
enum { MA_HATS = 0, MA_MASS = 1, MA_FACE = 2 };
cudaError_t multi_adj_launch(const Launchers &L, const void *basis, int nu, int nv, int kind,
                             const std::vector<AdjArgs> &args, cudaStream_t st) {
  const int TPW = 32 / (qhigh(nu, nv) / 2 + (qhigh(nu, nv) & 1));
  const int tile = kind == MA_MASS ? (CHEB_THREADS / 32) * TPW : ADJ_THREADS;
  const int n = (int)args.size();
  for (int c0 = 0; c0 < n; c0 += MultiAdj::cap) {
    const int m = std::min(n - c0, MultiAdj::cap);
    MultiAdj P;
    P.n = m;
    P.tile = tile;
    P.first[0] = 0;
    for (int x = 0; x < m; ++x) {
      P.a[x] = args[c0 + x];
      P.first[x + 1] = P.first[x] + (P.a[x].F.E + tile - 1) / tile;
    }
    const cudaError_t e = kind == MA_HATS ? L.adj_hats_m(basis, P, 0, st)
                          : kind == MA_MASS ? L.adj_mass_m(basis, P, 0, st)
                                            : L.adj_face_m(basis, P, 0, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// out_i = a x_i + b y_i (+ z_i) over the instances of a group (y, z may be null)
cudaError_t multi_lincomb(const std::vector<LinPtrs> &p, double a, double b, cudaStream_t st) {
  for (size_t c0 = 0; c0 < p.size(); c0 += LIN_CAP) {
    LinMulti L;
    L.n = (int)std::min(p.size() - c0, (size_t)LIN_CAP);
    L.a = a;
    L.b = b;
    size_t most = 1;
    for (int x = 0; x < L.n; ++x) {
      L.p[x] = p[c0 + x];
      most = std::max(most, L.p[x].n);
    }
    const unsigned gx = (unsigned)std::min<size_t>((most + 255) / 256, 152 * 16 / std::max(1, L.n) + 1);
    k_lincomb_m<<<dim3(gx, L.n), 256, 0, st>>>(L);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---- a group of workspaces advanced together by multi-instance launches: the same degrees,
//      coefficient kernels, mass solver and 1D operators; everything of the group runs on the first
//      workspace's stream while a StreamGuard holds the others on it
struct StreamGuard {
  std::vector<wedg_ws *> ws;
  std::vector<cudaStream_t> own;
  explicit StreamGuard(const std::vector<wedg_ws *> &g) : ws(g) {
    for (wedg_ws *w : ws) own.push_back(w->stream);
    for (wedg_ws *w : ws) w->stream = ws[0]->stream;
  }
  ~StreamGuard() {
    for (size_t i = 0; i < ws.size(); ++i) ws[i]->stream = own[i];
  }
};

bool same_kernels(const wedg_ws *a, const wedg_ws *b) {
  return a->nu == b->nu && a->nv == b->nv && a->fast == b->fast && a->cfg.mass_solver == b->cfg.mass_solver &&
         a->basis == b->basis;
}

// One RHS evaluation (k_prep, k_stage, mass solve) of every workspace of a group, each with its
// own Fields and StageIO; one workspace: enqueue_stage. Advances the bin parities as enqueue_stage.
int group_stage(const std::vector<wedg_ws *> &G, const std::vector<StageIO> &S, const std::vector<Fields> &F) {
  if (G.size() == 1) return enqueue_stage(G[0], S[0], &F[0]);
  std::vector<StageArgs> args(G.size());
  for (size_t i = 0; i < G.size(); ++i) {
    args[i].F = F[i];
    args[i].S = S[i];
    args[i].S.parity = G[i]->parity;
    G[i]->parity = 1 - G[i]->parity;
    G[i]->stats.kernel_launches += 3;
    G[i]->stats.element_stages += G[i]->E;
  }
  wedg_ws *w = G[0];
  auto all = [](int, int total) { return total; };
  for (int kind : {MK_PREP, MK_STAGE, MK_MASS}) {
    const cudaError_t e = multi_stage_launch(w->L, w->basis.data(), w->nu, w->nv, w->fast, kind, args,
                                             kind == MK_PREP ? w->prep_threads : w->mass_threads, w->stream, all);
    if (e != cudaSuccess) return cuda_fail(w, e, "multi-instance launch");
  }
  return WEDG_OK;
}

// One RK4 step of every workspace of a group on its state (u[i], v[i]) at time t
int group_rk4(const std::vector<wedg_ws *> &G, double *const *u, double *const *v, double t, double dt,
              int stop_nonfinite) {
  if (G.size() == 1) return enqueue_rk4(G[0], u[0], v[0], t, dt, stop_nonfinite);
  const int n = (int)G.size();
  std::vector<StageIO> S(n);
  std::vector<Fields> F(n);
  for (int s = 0; s < 4; ++s) {
    for (int i = 0; i < n; ++i) {
      S[i] = rk4_stage_io(G[i], u[i], v[i], s, t, dt, nullptr, 0, nullptr, nullptr);
      F[i] = G[i]->F;
    }
    const int rc = group_stage(G, S, F);
    if (rc) return rc;
  }
  wedg_ws *w = G[0];
  if (w->cfg.mass_solver == WEDG_CG) {
    for (int i = 0; i < n; ++i) {
      const int nU = G[i]->E * G[i]->nu * G[i]->nu, nV = G[i]->E * G[i]->nv * G[i]->nv;
      k_rk4_final<<<std::min((nU + nV + 255) / 256, 152 * 8), 256, 0, w->stream>>>(
          nU, nV, u[i], v[i], G[i]->accu, G[i]->accv, dt / 6.0, G[i]->F.err, G[i]->F.nonfinite);
      G[i]->stats.kernel_launches += 1;
    }
  }
  for (int c0 = 0; c0 < n; c0 += LIN_CAP) {
    StepMulti P;
    P.n = std::min(n - c0, LIN_CAP);
    P.stop_nonfinite = stop_nonfinite;
    for (int x = 0; x < P.n; ++x) {
      wedg_ws *g = G[c0 + x];
      P.f[x] = StepFlagsP{g->F.err, g->F.nonfinite, g->steps_done};
      g->stats.kernel_launches += 1;
    }
    k_step_done_p<<<1, LIN_CAP, 0, w->stream>>>(P);
  }
  CK(w, cudaGetLastError());
  return WEDG_OK;
}

// The transpose of one RHS evaluation of every workspace of a group (enqueue_adjoint_core for
// each): Fs, S the forward evaluation's data, lam the weights, g the gradients (and gpar the
// per-element coefficient gradients, or null for all)
int group_adjoint_core(const std::vector<wedg_ws *> &G, const std::vector<Fields> &Fs, const std::vector<StageIO> &S,
                       const std::vector<const double *> &lam_u, const std::vector<const double *> &lam_v,
                       const std::vector<double *> &gu, const std::vector<double *> &gv,
                       const std::vector<double *> &gpar) {
  const int n = (int)G.size();
  if (n == 1) return enqueue_adjoint_core(G[0], Fs[0], S[0], lam_u[0], lam_v[0], gu[0], gv[0], gpar[0]);
  wedg_ws *w = G[0];
  auto all = [](int, int total) { return total; };
  std::vector<StageArgs> sa(n);
  std::vector<AdjArgs> aa(n);
  cudaError_t e;
  // μ = M(v)⁻¹ λ_v on the Chebyshev data of the states
  for (int i = 0; i < n; ++i) {
    sa[i].F = Fs[i];
    sa[i].F.mrhs = const_cast<double *>(lam_v[i]);
    sa[i].S = S[i];
    sa[i].S.mode = OUT_RHS;
    sa[i].S.vt = G[i]->adj_mu;
  }
  if ((e = multi_stage_launch(w->L, w->basis.data(), w->nu, w->nv, w->fast, MK_MASS, sa, w->mass_threads, w->stream,
                              all)) != cudaSuccess)
    return cuda_fail(w, e, "multi-instance launch");
  // ν = A_e⁻¹ λ_u
  for (int i = 0; i < n; ++i) {
    sa[i].F = Fs[i];
    sa[i].S = S[i];
    sa[i].S.mode = OUT_ADJ_USOLVE;
    sa[i].S.xu = lam_u[i];
    sa[i].S.ut = G[i]->adj_nu;
  }
  if ((e = multi_stage_launch(w->L, w->basis.data(), w->nu, w->nv, w->fast, MK_STAGE, sa, 0, w->stream, all)) !=
      cudaSuccess)
    return cuda_fail(w, e, "multi-instance launch");
  for (int i = 0; i < n; ++i) {
    wedg_ws *g = G[i];
    aa[i].F = Fs[i];
    aa[i].S = S[i];
    aa[i].A = AdjIO{g->adj_mu, g->adj_nu, g->adj_nus, S[i].vt, g->adj_hat, gu[i], gv[i], S[i].xv,
                    gpar[i] ? gpar[i] + 2 * (size_t)g->E : nullptr};
    aa[i].gc2 = gpar[i];
    aa[i].gal = gpar[i] ? gpar[i] + g->E : nullptr;
    aa[i].gbe = gpar[i] ? gpar[i] + 2 * (size_t)g->E : nullptr;
  }
  if ((e = multi_adj_launch(w->L, w->basis.data(), w->nu, w->nv, MA_HATS, aa, w->stream)) != cudaSuccess)
    return cuda_fail(w, e, "multi-instance launch");
  // the volume transposes: the volume terms of the state (-(h²/4) ν, μ)
  for (int i = 0; i < n; ++i) {
    sa[i].F = Fs[i];
    sa[i].S = S[i];
    sa[i].S.mode = OUT_ADJ_VOLUME;
    sa[i].S.xu = G[i]->adj_nus;
    sa[i].S.xv = G[i]->adj_mu;
    sa[i].S.vt = gv[i];
    sa[i].S.ut = gu[i];
  }
  if ((e = multi_stage_launch(w->L, w->basis.data(), w->nu, w->nv, w->fast, MK_STAGE, sa, 0, w->stream, all)) !=
      cudaSuccess)
    return cuda_fail(w, e, "multi-instance launch");
  if ((e = multi_adj_launch(w->L, w->basis.data(), w->nu, w->nv, MA_MASS, aa, w->stream)) != cudaSuccess ||
      (e = multi_adj_launch(w->L, w->basis.data(), w->nu, w->nv, MA_FACE, aa, w->stream)) != cudaSuccess)
    return cuda_fail(w, e, "multi-instance launch");
  for (wedg_ws *g : G) g->stats.kernel_launches += 6;
  CK(w, cudaGetLastError());
  return WEDG_OK;
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

namespace {

// The forward run of a reverse sweep for every workspace of a group (wedg_rk4_adjoint_forward;
// several workspaces: their RK4 steps as multi-instance launches, in lockstep)
int adjoint_forward_group(const std::vector<wedg_ws *> &G, const double *const *u0, const double *const *v0,
                          double t0, double dt, int64_t nsteps, int64_t every, double *const *uT, double *const *vT,
                          int where) {
  PointTraces point_traces(G);
  const int n = (int)G.size();
  if (nsteps < 0 || every < 1) return argument_error(G[0], "nsteps must be ≥ 0 and the checkpoint interval ≥ 1");
  const int64_t nchk = nsteps ? (nsteps + every - 1) / every : 0;
  const int64_t seg = std::min<int64_t>(every, std::max<int64_t>(nsteps, 1));
  int rc;
  for (wedg_ws *ws : G) {
    const size_t nU = (size_t)ws->E * ws->nu * ws->nu, nV = (size_t)ws->E * ws->nv * ws->nv, nn = nU + nV;
    if ((rc = adjoint_buffers(ws))) return rc;
    // buffers: a state is u followed by v (nn doubles)
    if (!ws->rk_lam) {
      if ((rc = dalloc(ws, &ws->rk_lam, nn)) || (rc = dalloc(ws, &ws->rk_acc, nn)) ||
          (rc = dalloc(ws, &ws->rk_kbar, nn)) || (rc = dalloc(ws, &ws->rk_g, nn)) || (rc = dalloc(ws, &ws->rk_y, nn)) ||
          (rc = dalloc(ws, &ws->rk_par, 3 * (size_t)ws->E)))
        return rc;
    }
    while (ws->rk_chk_n < nchk) {
      double *p;
      if ((rc = dalloc(ws, &p, nn))) return rc;
      ws->rk_chk.push_back(p);
      ++ws->rk_chk_n;
    }
    while (ws->rk_seg_n < 4 * seg) {
      double *p;
      if ((rc = dalloc(ws, &p, nn))) return rc;
      ws->rk_seg.push_back(p);
      ++ws->rk_seg_n;
    }
  }
  StreamGuard guard(G);
  cudaStream_t st = G[0]->stream;
  const cudaMemcpyKind in = where == WEDG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  std::vector<double *> yu(n), yv(n);
  for (int i = 0; i < n; ++i) {
    wedg_ws *ws = G[i];
    const size_t nU = (size_t)ws->E * ws->nu * ws->nu, nV = (size_t)ws->E * ws->nv * ws->nv;
    yu[i] = ws->rk_y;
    yv[i] = ws->rk_y + nU;
    CK(ws, cudaMemcpyAsync(yu[i], u0[i], sizeof(double) * nU, in, st));
    CK(ws, cudaMemcpyAsync(yv[i], v0[i], sizeof(double) * nV, in, st));
    ws->rk_t.assign(nsteps + 1, t0);
    for (int64_t k = 0; k < nsteps; ++k) ws->rk_t[k + 1] = ws->rk_t[k] + dt;
    if ((rc = reset_flags(ws))) return rc;
  }
  const std::vector<double> &t = G[0]->rk_t;
  for (int64_t k = 0; k < nsteps; ++k) {
    if (k % every == 0)
      for (wedg_ws *ws : G)
        CK(ws, cudaMemcpyAsync(ws->rk_chk[k / every], ws->rk_y,
                               sizeof(double) * ws->E * (ws->nu * ws->nu + ws->nv * ws->nv), cudaMemcpyDeviceToDevice,
                               st));
    if ((rc = group_rk4(G, yu.data(), yv.data(), t[k], dt, 1))) return rc;
  }
  CK(G[0], cudaGetLastError());
  int first = WEDG_OK;
  for (wedg_ws *ws : G) {
    const int64_t launches = ws->stats.kernel_launches;
    rc = collect(ws);
    ws->stats.kernel_launches = launches;
    if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
    if (rc != WEDG_OK && first == WEDG_OK) first = rc;
    if (!ws->stats.finite) return argument_error(ws, "the forward run is not finite");
  }
  const cudaMemcpyKind out = where == WEDG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  for (int i = 0; i < n; ++i) {
    wedg_ws *ws = G[i];
    const size_t nU = (size_t)ws->E * ws->nu * ws->nu, nV = (size_t)ws->E * ws->nv * ws->nv;
    if (uT[i]) CK(ws, cudaMemcpy(uT[i], yu[i], sizeof(double) * nU, out));
    if (vT[i]) CK(ws, cudaMemcpy(vT[i], yv[i], sizeof(double) * nV, out));
    ws->rk_dt = dt;
    ws->rk_nsteps = nsteps;
    ws->rk_every = every;
    ws->rk_ready = true;
  }
  return first;
}

// The reverse sweep of every workspace of a group after its forward run (wedg_rk4_adjoint_reverse;
// several workspaces: the forward runs must have the same steps, dt and checkpoint interval, and
// every stage's transpose runs as multi-instance launches over the group, which needs the stage
// data of one segment of every workspace kept at once; when that does not fit the allowance the
// workspaces are reversed one after the other)
int adjoint_reverse_group(const std::vector<wedg_ws *> &G, const double *const *lam_u, const double *const *lam_v,
                          double *const *gu, double *const *gv, double *const *g_c2, double *const *g_alpha,
                          double *const *g_beta, int where) {
  PointTraces point_traces(G);
  const int n = (int)G.size();
  for (wedg_ws *ws : G) ws->stats.kernel_launches = 0;
  const bool params = g_c2[0] || g_alpha[0] || g_beta[0];
  for (int i = 0; i < n; ++i) {
    wedg_ws *ws = G[i];
    if (!ws->rk_ready)
      return argument_error(ws, "no forward run with checkpoints (wedg_rk4_adjoint_forward) to reverse");
    if (!lam_u[i] || !lam_v[i] || !gu[i] || !gv[i]) return argument_error(ws, "null pointer");
    const bool p = g_c2[i] || g_alpha[i] || g_beta[i];
    if (p != params || (p && !(g_c2[i] && g_alpha[i] && g_beta[i])))
      return argument_error(ws, "give all three parameter gradients or none");
    if (p && (!ws->fast || !ws->cfg.src_on || ws->cfg.mms_on))
      return argument_error(ws, "parameter gradients need source mode and c², α, β constant on each element");
    if (ws->rk_nsteps != G[0]->rk_nsteps || ws->rk_every != G[0]->rk_every || ws->rk_dt != G[0]->rk_dt)
      return argument_error(ws, "the forward runs of a group need the same steps, dt and checkpoint interval");
  }
  const int64_t nsteps = G[0]->rk_nsteps, every = G[0]->rk_every;
  const int64_t nchk = nsteps ? (nsteps + every - 1) / every : 0;
  const double dt = G[0]->rk_dt;
  // keep the forward data of every stage of a segment when it fits the memory allowance
  const int64_t seg = std::min<int64_t>(every, std::max<int64_t>(nsteps, 1));
  size_t need = 0, have = 0, allow = 0;
  bool bounded = true;
  for (wedg_ws *ws : G) {
    need += (size_t)(4 * seg) * stage_data_bytes(ws);
    have += ws->rk_keep.size() * stage_data_bytes(ws);
    if (ws->adj_mem >= 0) allow += (size_t)ws->adj_mem;
    else bounded = false;
  }
  // with room for two segments' data, the forward data of the next segment (back in time) is
  // recomputed on a second stream while the present segment is reversed: the two overlap on a GPU
  // that one problem of this size does not fill
  size_t extra = 0;                            // the second set's stage states and the recompute's buffers
  for (wedg_ws *ws : G)
    extra += sizeof(double) * (size_t)ws->E * (ws->nu * ws->nu + ws->nv * ws->nv) * (4 * seg + 2);
  bool keep, pipe;
  if (!bounded) {
    size_t fr = 0, tot = 0;
    const bool info = cudaMemGetInfo(&fr, &tot) == cudaSuccess;
    keep = info && need <= (fr + have) / 2;
    pipe = info && nchk > 1 && 2 * need + extra <= (fr + have) / 2;
  } else {
    keep = need <= allow;
    pipe = nchk > 1 && 2 * need + extra <= allow;
  }
  if (n > 1 && !keep) {
    // one after the other, each with its own allowance
    for (int i = 0; i < n; ++i) {
      const int rc = adjoint_reverse_group({G[i]}, lam_u + i, lam_v + i, gu + i, gv + i, g_c2 + i, g_alpha + i,
                                           g_beta + i, where);
      if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
    }
    return WEDG_OK;
  }
  int rc;
  StreamGuard guard(G);
  cudaStream_t st = G[0]->stream;               // the reverse sweep
  cudaStream_t sr = st;                         // the recompute (its own stream when pipelined)
  const int nset = pipe ? 2 : 1;
  const cudaMemcpyKind in = where == WEDG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  std::vector<size_t> nU(n), nV(n), nn(n);
  for (int i = 0; i < n; ++i) {
    wedg_ws *ws = G[i];
    nU[i] = (size_t)ws->E * ws->nu * ws->nu;
    nV[i] = (size_t)ws->E * ws->nv * ws->nv;
    nn[i] = nU[i] + nV[i];
    CK(ws, cudaMemcpyAsync(ws->rk_lam, lam_u[i], sizeof(double) * nU[i], in, st));
    CK(ws, cudaMemcpyAsync(ws->rk_lam + nU[i], lam_v[i], sizeof(double) * nV[i], in, st));
    if (params) CK(ws, cudaMemsetAsync(ws->rk_par, 0, sizeof(double) * 3 * ws->E, st));
    if ((rc = reset_flags(ws))) return rc;
    if (keep) {
      const size_t E = ws->E;
      const size_t nd = (size_t)ws->nu * ws->nu + ws->nv * ws->nv + 12 * ws->nq + ws->qh * ws->qh + 2;
      while ((int64_t)ws->rk_keep.size() < nset * 4 * seg) {
        wedg_ws::StageData d;
        double *bd;
        int *ib;
        if ((rc = dalloc(ws, &bd, nd * E)) || (rc = dalloc(ws, &ib, E * (1 + NBIN) + 2 * NBIN + 4))) return rc;
        d.k = bd;
        d.tr = d.k + nn[i];
        d.G = d.tr + 12 * (size_t)ws->nq * E;
        d.th = d.G + (size_t)ws->qh * ws->qh * E;
        d.de = d.th + E;
        d.nst = ib;
        d.bins = ib + E;
        d.bin_count = ib + E * (1 + NBIN);
        d.nmax = d.bin_count + 2 * NBIN;
        ws->rk_keep.push_back(d);
      }
      while (ws->rk_seg_n < nset * 4 * seg) {
        double *p;
        if ((rc = dalloc(ws, &p, nn[i]))) return rc;
        ws->rk_seg.push_back(p);
        ++ws->rk_seg_n;
      }
      if (pipe && !ws->rk_ry && ((rc = dalloc(ws, &ws->rk_ry, nn[i])) || (rc = dalloc(ws, &ws->rk_racc, nn[i]))))
        return rc;
    }
  }
  // streams and events of the pipeline (destroyed on every return path)
  struct PipeRes {
    cudaStream_t s = nullptr;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    ~PipeRes() {
      if (s) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
      }
      for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
    }
  } pr;
  cudaEvent_t *ev_rec = pr.ev, *ev_adj = pr.ev + 2, &ev_start = pr.ev[4];
  if (pipe) {
    CK(G[0], cudaStreamCreateWithFlags(&pr.s, cudaStreamNonBlocking));
    for (cudaEvent_t &e : pr.ev) CK(G[0], cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    sr = pr.s;
    CK(G[0], cudaEventRecord(ev_start, st));    // the recompute starts after this call's set-up
    CK(G[0], cudaStreamWaitEvent(sr, ev_start, 0));
  }
  auto on = [&](cudaStream_t x) {
    for (wedg_ws *ws : G) ws->stream = x;
  };
  // out_i = a x_i + b y_i (+ z_i) for the group on stream x; out etc. give the instance's buffers
  auto lin_on = [&](cudaStream_t x, auto out, double a, auto xs, double b, auto y, auto z) -> int {
    std::vector<LinPtrs> p(n);
    for (int i = 0; i < n; ++i) {
      p[i] = LinPtrs{nn[i], out(i), xs(i), y(i), z(i)};
      G[i]->stats.kernel_launches += 1;
    }
    const cudaError_t e = multi_lincomb(p, a, b, x);
    return e == cudaSuccess ? WEDG_OK : cuda_fail(G[0], e, "k_lincomb_m");
  };
  auto none = [](int) -> const double * { return nullptr; };
  const double ca[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};
  const double cb[4] = {0.5 * dt, 0.5 * dt, dt, 0.0};
  const double cs[3] = {0.5 * dt, 0.5 * dt, dt};
  std::vector<StageIO> S(n);
  std::vector<Fields> F(n);
  std::vector<const double *> lu(n), lv(n);
  std::vector<double *> ggu(n), ggv(n), gpar(n);
  // ---- the forward data of segment c into set `set` (stream sr): every stage's RHS evaluated
  //      with its outputs and data kept, and the RK4 combinations: Y1 = y, Y_{s+1} = y + c_s K_s,
  //      y ← y + dt/6 (K1 + 2K2 + 2K3 + K4)
  auto recompute = [&](int64_t c, int set) -> int {
    const int64_t k0 = c * every, k1 = std::min(nsteps, k0 + every);
    const size_t base = (size_t)set * 4 * seg;
    on(sr);
    auto y = [&](int i) { return pipe ? G[i]->rk_ry : G[i]->rk_y; };
    auto yc = [&](int i) -> const double * { return pipe ? G[i]->rk_ry : G[i]->rk_y; };
    auto acc = [&](int i) { return pipe ? G[i]->rk_racc : G[i]->rk_acc; };
    auto accc = [&](int i) -> const double * { return pipe ? G[i]->rk_racc : G[i]->rk_acc; };
    for (int i = 0; i < n; ++i)
      CK(G[i], cudaMemcpyAsync(y(i), G[i]->rk_chk[c], sizeof(double) * nn[i], cudaMemcpyDeviceToDevice, sr));
    for (int64_t k = k0; k < k1; ++k) {
      const size_t q = base + 4 * (k - k0);
      for (int i = 0; i < n; ++i)
        CK(G[i], cudaMemcpyAsync(G[i]->rk_seg[q], y(i), sizeof(double) * nn[i], cudaMemcpyDeviceToDevice, sr));
      for (int s = 0; s < 4; ++s) {
        for (int i = 0; i < n; ++i) {
          wedg_ws *ws = G[i];
          const std::vector<double> &t = ws->rk_t;
          const double ts[4] = {t[k], t[k] + 0.5 * dt, t[k] + 0.5 * dt, t[k] + dt};
          wedg_ws::StageData &d = ws->rk_keep[q + s];
          const double *Y = ws->rk_seg[q + s];
          S[i] = StageIO{};
          S[i].xu = Y; S[i].xv = Y + nU[i];
          stage_factors(ws, ts[s], S[i]);
          S[i].mode = OUT_RHS;
          S[i].ut = d.k;
          S[i].vt = d.k + nU[i];
          CK(ws, cudaMemsetAsync(d.bin_count, 0, (2 * NBIN + 3) * sizeof(int), sr));   // and d.nmax
          d.parity = ws->parity;
          F[i] = kept_fields(ws, d);
        }
        int r;
        if ((r = group_stage(G, S, F))) return r;
        if (s < 3 && (r = lin_on(sr, [&](int i) { return G[i]->rk_seg[q + s + 1]; }, cs[s],
                                 [&](int i) -> const double * { return G[i]->rk_keep[q + s].k; }, 1.0, yc, none)))
          return r;
      }
      auto K = [&](int s) { return [&, s](int i) -> const double * { return G[i]->rk_keep[q + s].k; }; };
      int r;
      if ((r = lin_on(sr, acc, 2.0, K(1), 1.0, K(0), none)) || (r = lin_on(sr, acc, 2.0, K(2), 1.0, K(3), accc)) ||
          (r = lin_on(sr, y, dt / 6.0, accc, 1.0, yc, none)))
        return r;
    }
    return WEDG_OK;
  };
  // ---- the reverse steps of segment c from the data of set `set` (or, for one workspace without
  //      room to keep data, the stage states of a recompute and each stage's forward RHS evaluated
  //      again), on stream st
  auto reverse = [&](int64_t c, int set) -> int {
    const int64_t k0 = c * every, k1 = std::min(nsteps, k0 + every);
    const size_t base = (size_t)set * 4 * seg;
    int r;
    on(st);
    if (!keep) {
      wedg_ws *ws = G[0];
      CK(ws, cudaMemcpyAsync(ws->rk_y, ws->rk_chk[c], sizeof(double) * nn[0], cudaMemcpyDeviceToDevice, st));
      for (int64_t k = k0; k < k1; ++k) {
        double *su[4], *sv[4];
        for (int s = 0; s < 4; ++s) {
          su[s] = ws->rk_seg[4 * (k - k0) + s];
          sv[s] = su[s] + nU[0];
        }
        if ((r = enqueue_rk4(ws, ws->rk_y, ws->rk_y + nU[0], ws->rk_t[k], dt, 1, nullptr, 0, su, sv))) return r;
      }
    }
    for (int64_t k = k1 - 1; k >= k0; --k) {
      // K̄_s = ca[s] λ + cb[s] Ȳ_{s+1}, Ȳ = Jᵀ K̄ at the stage state: y_{n+1} = y + dt/6 (K1 + 2K2 +
      // 2K3 + K4), Y2 = y + dt/2 K1, Y3 = y + dt/2 K2, Y4 = y + dt K3
      const size_t q = base + 4 * (k - k0);
      for (int s = 3; s >= 0; --s) {
        if ((r = lin_on(st, [&](int i) { return G[i]->rk_kbar; }, ca[s],
                        [&](int i) -> const double * { return G[i]->rk_lam; }, cb[s],
                        [&](int i) -> const double * { return s == 3 ? nullptr : G[i]->rk_g; }, none)))
          return r;
        for (int i = 0; i < n; ++i) {
          wedg_ws *ws = G[i];
          lu[i] = ws->rk_kbar;
          lv[i] = ws->rk_kbar + nU[i];
          ggu[i] = ws->rk_g;
          ggv[i] = ws->rk_g + nU[i];
          gpar[i] = params ? ws->rk_par : nullptr;
        }
        if (keep) {
          for (int i = 0; i < n; ++i) {
            wedg_ws *ws = G[i];
            const std::vector<double> &t = ws->rk_t;
            const double ts[4] = {t[k], t[k] + 0.5 * dt, t[k] + 0.5 * dt, t[k] + dt};
            const wedg_ws::StageData &d = ws->rk_keep[q + s];
            const double *Y = ws->rk_seg[q + s];
            S[i] = StageIO{};
            S[i].xu = Y; S[i].xv = Y + nU[i];
            stage_factors(ws, ts[s], S[i]);
            S[i].parity = d.parity;
            S[i].ut = d.k;
            S[i].vt = d.k + nU[i];
            F[i] = kept_fields(ws, d);
          }
          r = group_adjoint_core(G, F, S, lu, lv, ggu, ggv, gpar);
        } else {
          wedg_ws *ws = G[0];
          const std::vector<double> &t = ws->rk_t;
          const double ts[4] = {t[k], t[k] + 0.5 * dt, t[k] + 0.5 * dt, t[k] + dt};
          const double *Y = ws->rk_seg[4 * (k - k0) + s];
          r = enqueue_rhs_adjoint(ws, Y, Y + nU[0], ts[s], lu[0], lv[0], ggu[0], ggv[0], gpar[0]);
        }
        if (r) return r;
        if ((r = lin_on(st, [&](int i) { return G[i]->rk_acc; }, 1.0,
                        [&](int i) -> const double * { return s == 3 ? G[i]->rk_lam : G[i]->rk_acc; }, 1.0,
                        [&](int i) -> const double * { return G[i]->rk_g; }, none)))
          return r;
      }
      for (wedg_ws *ws : G) std::swap(ws->rk_lam, ws->rk_acc);
    }
    return WEDG_OK;
  };
  // ---- reverse pass, segment by segment
  if (pipe) {
    // set c % 2 holds segment c; the recompute of c - 1 into the other set waits for the reverse
    // of c + 1 (which read it), the reverse of c for the recompute of c
    if ((rc = recompute(nchk - 1, (int)((nchk - 1) % 2)))) return rc;
    CK(G[0], cudaEventRecord(ev_rec[(nchk - 1) % 2], sr));
    for (int64_t c = nchk - 1; c >= 0; --c) {
      const int set = (int)(c % 2);
      if (c >= 1) {
        CK(G[0], cudaStreamWaitEvent(sr, ev_adj[1 - set], 0));
        if ((rc = recompute(c - 1, 1 - set))) return rc;
        CK(G[0], cudaEventRecord(ev_rec[1 - set], sr));
      }
      CK(G[0], cudaStreamWaitEvent(st, ev_rec[set], 0));
      if ((rc = reverse(c, set))) return rc;
      CK(G[0], cudaEventRecord(ev_adj[set], st));
    }
  } else {
    for (int64_t c = nchk - 1; c >= 0; --c) {
      if (keep && (rc = recompute(c, 0))) return rc;
      if ((rc = reverse(c, 0))) return rc;
    }
  }
  on(st);
  CK(G[0], cudaGetLastError());
  int first = WEDG_OK;
  const cudaMemcpyKind out = where == WEDG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  for (int i = 0; i < n; ++i) {
    wedg_ws *ws = G[i];
    const int64_t launches = ws->stats.kernel_launches;
    rc = collect(ws);
    ws->stats.kernel_launches = launches;
    if (rc != WEDG_OK && first == WEDG_OK) first = rc;
    CK(ws, cudaMemcpy(gu[i], ws->rk_lam, sizeof(double) * nU[i], out));
    CK(ws, cudaMemcpy(gv[i], ws->rk_lam + nU[i], sizeof(double) * nV[i], out));
    if (params) {
      CK(ws, cudaMemcpy(g_c2[i], ws->rk_par, sizeof(double) * ws->E, out));
      CK(ws, cudaMemcpy(g_alpha[i], ws->rk_par + ws->E, sizeof(double) * ws->E, out));
      CK(ws, cudaMemcpy(g_beta[i], ws->rk_par + 2 * ws->E, sizeof(double) * ws->E, out));
    }
  }
  return first;
}

}  // namespace

namespace wedg {

// Step bookkeeping of many instances in one launch (the batched form): thread i does
// k_step_done's work for instance i
struct StepFlags {
  unsigned long long *err;
  const unsigned int *nonfinite;
  long long *steps_done;
};
__global__ void k_step_done_m(int n, const StepFlags *f, int stop_nonfinite) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const StepFlags x = f[i];
  if (*x.err != ERR_NONE) return;
  *x.steps_done += 1;
  if (stop_nonfinite && *x.nonfinite) *x.err = (3ull << ERR_CLASS_SHIFT);
}

// k_rk4_final of many CG instances in one launch: blockIdx.y is the instance
struct FinalArgs {
  int n_u, n_v;
  double *u, *v;
  const double *accu, *accv;
  double c;
  const unsigned long long *err;
  unsigned int *nonfinite;
};
__global__ void k_rk4_final_m(const FinalArgs *a) {
  const FinalArgs A = a[blockIdx.y];
  if (*(volatile const unsigned long long *)A.err != ERR_NONE) return;
  bool fin = true;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n_u + A.n_v; i += gridDim.x * blockDim.x) {
    if (i < A.n_u) {
      const double x = A.u[i] + A.c * A.accu[i];
      A.u[i] = x;
      fin = fin && isfinite(x);
    } else {
      const int l = i - A.n_u;
      const double x = A.v[l] + A.c * A.accv[l];
      A.v[l] = x;
      fin = fin && isfinite(x);
    }
  }
  if (!fin) atomicOr(A.nonfinite, 1u);
}

}  // namespace wedg

namespace {

// Instances of a batch that run the same kernels -- the same degrees, coefficient kernels
// (constant per element or not), mass solver and 1D operators -- and share one multi-instance
// launch per kernel and stage, with the bucket's launch shape: threads per block of k_prep and of
// the mass solves, and `persist` (0: one block per virtual block; p > 0: a persistent grid of p
// times the blocks the SMs hold at once). With `split` the bucket's instances are launched one by
// one instead, each on its own stream forked from the bucket's (the single-instance kernels).
struct BatchBucket {
  std::vector<int> ids;   // instances, largest mesh first
  Launchers L;
  std::vector<char> basis;
  int nu = 0, nv = 0;
  bool fast = false, cg = false;
  int prep_threads = 128, mass_threads = CHEB_THREADS, persist = 0;
  bool split = true;   // the default: faster than the merged launches on the mixed batches measured
  cudaStream_t st = nullptr;
  cudaEvent_t join = nullptr, fork = nullptr;
  StepFlags *d_flags = nullptr;   // per instance of the bucket, for k_step_done_m
  FinalArgs *d_final = nullptr;   // per instance, for k_rk4_final_m (CG)
};

}  // namespace

// A batch of workspaces advanced by one replayed CUDA graph per step (wedg_batch_*): per bucket
// of instances, one launch per kernel and stage covering all of its instances
struct wedg_batch {
  std::vector<wedg_ws *> ws;
  std::vector<BatchBucket> buckets;
  int nsm = 152;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  cudaEvent_t half_done[2] = {nullptr, nullptr};   // the host half of the tables may be refilled
  // graph[0]: one RK4 step of every instance; graph[1]: kBatchGraphSteps steps, in which each
  // instance (or merged bucket) goes on to its next step without waiting for the others
  cudaGraph_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  // what the captured graphs were made for
  std::vector<double *> gu, gv;
  std::vector<double> gdt;
  std::vector<int64_t> step_launches;               // per instance: its kernel launches in one step
  BatchFlagPtrs *d_flagp = nullptr;                 // per instance: its flags (k_batch_reset, k_batch_read)
  BatchFlagVals *d_flagv = nullptr, *h_flagv = nullptr;   // their values after a call (h_flagv pinned)
  double *d_tf_all = nullptr;                       // the instances' factor tables, instance after instance
  int gstop = -1;
  int64_t shape_gen = 0, gshape = -1;              // changes of the buckets' launch shapes
  // per instance: device factor table of 2 chunks (the kernels index it by step mod 2 chunks)
  std::vector<double *> d_tf;
  double *h_tf = nullptr;                           // pinned: 2 halves × instances × one chunk
  std::vector<void *> dmem;                         // device arrays of the buckets
  std::vector<cudaEvent_t> ijoin;                   // per instance: the end of its launches (split buckets)
  ~wedg_batch() {
    if (main) cudaStreamSynchronize(main);
    for (BatchBucket &k : buckets)
      if (k.st) cudaStreamSynchronize(k.st);
    for (int g = 0; g < 2; ++g) {
      if (exec[g]) cudaGraphExecDestroy(exec[g]);
      if (graph[g]) cudaGraphDestroy(graph[g]);
    }
    if (d_tf_all) cudaFree(d_tf_all);
    if (d_flagp) cudaFree(d_flagp);
    if (d_flagv) cudaFree(d_flagv);
    if (h_flagv) cudaFreeHost(h_flagv);
    for (void *p : dmem) cudaFree(p);
    if (h_tf) cudaFreeHost(h_tf);
    for (BatchBucket &k : buckets) {
      if (k.join) cudaEventDestroy(k.join);
      if (k.fork) cudaEventDestroy(k.fork);
      if (k.st) cudaStreamDestroy(k.st);
    }
    for (cudaEvent_t e : ijoin) cudaEventDestroy(e);
    for (cudaEvent_t e : half_done)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (main) cudaStreamDestroy(main);
  }
};

namespace {

// Physical blocks of a multi-instance launch of `total` virtual blocks: all of them, or with
// persist > 0 that many times the blocks the SMs hold at once (resident blocks per SM at 128
// threads, scaled for smaller blocks)
int bucket_grid(const wedg_batch *b, const BatchBucket &k, int total, int resident128, int threads) {
  if (k.persist <= 0) return total;
  const int cap = k.persist * b->nsm * resident128 * (128 / std::max(32, std::min(128, threads)));
  return std::min(total, std::max(cap, 1));
}

int enqueue_merged_step(wedg_batch *b, BatchBucket &k, double *const *u, double *const *v, const double *t,
                        const double *dt, int stop_nonfinite, bool tables, long long tf_n);

// Enqueue `steps` RK4 steps of every instance of bucket k on its stream: per stage, k_prep,
// k_stage and the mass solve as multi-instance launches (chunks of up to MultiStage::cap
// instances), then the last update of CG instances and the step bookkeeping. u, v, t, dt are
// indexed by instance (t is ignored with tables: the stage kernels then read their time factors
// from the instances' device tables d_tf, tf_n steps, at the instance's device step counter; without
// tables `steps` is 1). Advances each instance's bin parity as enqueue_stage does. A split bucket's
// instances run their steps one after another on their own streams, with no join between steps.
int enqueue_bucket_step(wedg_batch *b, BatchBucket &k, double *const *u, double *const *v, const double *t,
                        const double *dt, int stop_nonfinite, bool tables, long long tf_n, int steps = 1) {
  const int n = (int)k.ids.size();
  if (k.split) {
    // every instance on its own stream, forked from and joined to the bucket's
    cudaError_t e = cudaEventRecord(k.fork, k.st);
    for (int x = 0; x < n && e == cudaSuccess; ++x) {
      const int i = k.ids[x];
      wedg_ws *w = b->ws[i];
      e = cudaStreamWaitEvent(w->stream, k.fork, 0);
      if (e != cudaSuccess) break;
      const bool timing = w->timing;
      w->timing = false;
      const int pt = w->prep_threads, mt = w->mass_threads;
      w->prep_threads = k.prep_threads;
      w->mass_threads = k.mass_threads;
      int rc = WEDG_OK;
      for (int it = 0; it < steps && rc == WEDG_OK; ++it)
        rc = enqueue_rk4(w, u[i], v[i], tables ? 0.0 : t[i], dt[i], stop_nonfinite, tables ? b->d_tf[i] : nullptr,
                         tables ? tf_n : 0);
      w->prep_threads = pt;
      w->mass_threads = mt;
      w->timing = timing;
      if (rc) return rc;
      e = cudaEventRecord(b->ijoin[i], w->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(k.st, b->ijoin[i], 0);
    }
    if (e != cudaSuccess) return cuda_fail(b->ws[k.ids[0]], e, "split bucket launch");
    return WEDG_OK;
  }
  for (int it = 0; it < steps; ++it) {
    const int rc = enqueue_merged_step(b, k, u, v, t, dt, stop_nonfinite, tables, tf_n);
    if (rc) return rc;
  }
  return WEDG_OK;
}

// One RK4 step of a merged bucket (see enqueue_bucket_step)
int enqueue_merged_step(wedg_batch *b, BatchBucket &k, double *const *u, double *const *v, const double *t,
                        const double *dt, int stop_nonfinite, bool tables, long long tf_n) {
  const int n = (int)k.ids.size();
  const int BT = stage_threads(k.nu, k.nv, k.fast);
  const int TPW = 32 / (qhigh(k.nu, k.nv) / 2 + (qhigh(k.nu, k.nv) & 1));
  const int mass_tile = (k.mass_threads / 32) * TPW;
  std::vector<StageArgs> args(n);
  for (int s = 0; s < 4; ++s) {
    for (int x = 0; x < n; ++x) {
      const int i = k.ids[x];
      wedg_ws *w = b->ws[i];
      StageIO S = rk4_stage_io(w, u[i], v[i], s, tables ? 0.0 : t[i], dt[i], tables ? b->d_tf[i] : nullptr,
                               tables ? tf_n : 0, nullptr, nullptr);
      S.parity = w->parity;
      w->parity = 1 - w->parity;
      args[x].F = w->F;
      args[x].S = S;
      w->stats.kernel_launches += 3;
      w->stats.element_stages += w->E;
    }
    for (int kind = 0; kind < 3; ++kind) {
      const int tile = kind == 0 ? k.prep_threads : kind == 1 ? BT : mass_tile;
      for (int c0 = 0; c0 < n; c0 += MultiStage::cap) {
        const int m = std::min(n - c0, MultiStage::cap);
        MultiStage P;
        P.n = m;
        P.tile = tile;
        P.first[0] = 0;
        for (int x = 0; x < m; ++x) {
          P.a[x] = args[c0 + x];
          P.first[x + 1] = P.first[x] + (P.a[x].F.E + tile - 1) / tile;
        }
        const int total = P.first[m];
        cudaError_t e;
        if (kind == 0)
          e = k.L.prep_m(k.basis.data(), P, bucket_grid(b, k, total, 3, k.prep_threads), k.prep_threads, k.st);
        else if (kind == 1)
          e = k.L.stage_m(k.basis.data(), P, bucket_grid(b, k, total, 2, 128), BT, k.st);
        else
          e = k.L.mass_m(k.basis.data(), P, bucket_grid(b, k, total, 3, k.mass_threads), k.mass_threads, k.st);
        if (e != cudaSuccess) return cuda_fail(b->ws[k.ids[0]], e, "multi-instance launch");
      }
    }
  }
  if (k.cg) {
    int most = 1;
    for (int i : k.ids) most = std::max(most, b->ws[i]->E * (b->ws[i]->nu * b->ws[i]->nu + b->ws[i]->nv * b->ws[i]->nv));
    k_rk4_final_m<<<dim3(std::min((most + 255) / 256, 152 * 8), n), 256, 0, k.st>>>(k.d_final);
  }
  k_step_done_m<<<(n + 127) / 128, 128, 0, k.st>>>(n, k.d_flags, stop_nonfinite);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(b->ws[k.ids[0]], e, "multi-instance launch");
  return WEDG_OK;
}

// The device arguments of k_rk4_final_m for the CG buckets (the state pointers and dt change).
// A captured graph reads them, so it is captured again after any upload.
int upload_final_args(wedg_batch *b, double *const *u, double *const *v, const double *dt) {
  b->gstop = -1;
  for (BatchBucket &k : b->buckets) {
    if (!k.cg) continue;
    const cudaError_t es = cudaStreamSynchronize(k.st);   // no launch of the bucket still reads them
    if (es != cudaSuccess) return cuda_fail(b->ws[k.ids[0]], es, "wedg_batch_rk4_steps");
    std::vector<FinalArgs> fa(k.ids.size());
    for (size_t x = 0; x < k.ids.size(); ++x) {
      const int i = k.ids[x];
      wedg_ws *w = b->ws[i];
      fa[x] = FinalArgs{w->E * w->nu * w->nu, w->E * w->nv * w->nv, u[i], v[i], w->accu, w->accv, dt[i] / 6.0,
                        w->F.err, w->F.nonfinite};
    }
    const cudaError_t e = cudaMemcpy(k.d_final, fa.data(), sizeof(FinalArgs) * fa.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(b->ws[k.ids[0]], e, "wedg_batch_rk4_steps");
  }
  return WEDG_OK;
}

}  // namespace

namespace {

// The checks of wedg_create on the configuration (and that a GPU is usable)
int validate_config(const wedg_config *cfg) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return WEDG_ERR_NO_DEVICE;
  const int N = cfg->N, nu = cfg->qu1, nv = cfg->qv1;
  if (N < 1 || nu < 2 || nu > MAXN || !(nv == nu || nv == nu - 1) || cfg->q_high != qhigh(nu, nv))
    return WEDG_ERR_ARGUMENT;
  if ((int64_t)N * N > (int64_t)1 << 30) return WEDG_ERR_ARGUMENT;
  for (int s = 0; s < 4; ++s)
    if (cfg->kind[s] < 0 || cfg->kind[s] > 3) return WEDG_ERR_ARGUMENT;
  if (cfg->mass_solver != WEDG_CHEBYSHEV && cfg->mass_solver != WEDG_CG) return WEDG_ERR_ARGUMENT;
  return WEDG_OK;
}

// A new workspace with the configuration's sizes and its 1D operators (with their mirror parities
// made exact); wedg_create and wedg_create_points then fill the device arrays
int create_begin(const wedg_config *cfg, const wedg_pre *pre, wedg_ws **out) {
  wedg_ws *ws = new wedg_ws();
  ws->cfg = *cfg;
  ws->N = cfg->N;
  ws->E = cfg->N * cfg->N;
  ws->nu = cfg->qu1;
  ws->nv = cfg->qv1;
  ws->nq = cfg->qu1;
  ws->qh = cfg->q_high;
  ws->F.N = ws->N;
  ws->F.E = ws->E;
  if (build_basis(cfg, pre, ws->bh)) {
    delete ws;
    return WEDG_ERR_ARGUMENT;
  }
  *out = ws;
  return WEDG_OK;
}

// The kernels of the workspace's degrees and coefficient family, and their 1D operators
int create_launchers(wedg_ws *ws, bool fast) {
  ws->fast = fast;
  ws->L = get_launchers(ws->nu, ws->nv, fast);
  if (!ws->L.prep) {
    wedg_destroy(ws);
    return WEDG_ERR_ARGUMENT;
  }
  ws->basis.resize(ws->L.basis_size);
  ws->L.pack(ws->bh, ws->basis.data());
  return WEDG_OK;
}

// The packed inverses of src/solver.jl:528-535 on the device from F.Cw (k_ainv); a stiffness that
// is not positive definite fails the creation (the workspace is destroyed)
int device_inverses(wedg_ws *ws, const wedg_pre *pre) {
  const int nu = ws->nu, nq = ws->nq, E = ws->E;
  const size_t nt = (size_t)nu * nu * (nu * nu + 1) / 2;
  const double *Pu = nullptr, *Su = nullptr;
  int rc;
  if ((rc = upload(ws, &Pu, std::vector<double>(pre->P_u, pre->P_u + (size_t)nq * nu))) ||
      (rc = upload(ws, &Su, std::vector<double>(pre->S_u, pre->S_u + (size_t)nq * nu)))) {
    wedg_destroy(ws);
    return rc;
  }
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
    k_ainv<<<E, 128, sm>>>(ws->F.Cw, E, nu, Pu, Su, ainv, bad);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpy(&nbad, bad, sizeof nbad, cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess || nbad) {
    wedg_destroy(ws);
    return ce != cudaSuccess ? WEDG_ERR_CUDA : WEDG_ERR_ARGUMENT;
  }
  ws->F.Ainv = ainv;
  return WEDG_OK;
}

// pre's boundary data (nq, N) -> [m + N i]
int upload_boundary(wedg_ws *ws, const wedg_pre *pre) {
  const int N = ws->N, nq = ws->nq;
  auto bd = [&](const double *a) {
    std::vector<double> o((size_t)nq * N);
    for (int m = 0; m < N; ++m)
      for (int i = 0; i < nq; ++i) o[m + (size_t)N * i] = a[i + nq * m];
    return o;
  };
  const double *sp[4] = {pre->bcB_sp, pre->bcT_sp, pre->bcL_sp, pre->bcR_sp};
  const double *spn[4] = {pre->bcB_spy, pre->bcT_spy, pre->bcL_spx, pre->bcR_spx};
  for (int s = 0; s < 4; ++s) {
    int rc;
    if ((rc = upload(ws, &ws->F.bsp[s], bd(sp[s]))) || (rc = upload(ws, &ws->F.bspn[s], bd(spn[s])))) {
      wedg_destroy(ws);
      return rc;
    }
  }
  return WEDG_OK;
}

// Whether the traces can be kept as modal end sums (Fields::modal): sets bit 0 of *flag when an
// interior face's coefficient values differ along the face, bit 1 when, with one-sided faces, its
// jump term is not zero (its projections are then needed). One thread per interior face: the
// horizontal faces (jf, k), jf = 1..N-1, then the vertical faces (j, kf), kf = 1..N-1, in the
// device layouts [jf + (N+1)(k + N i)] and [j + N(kf + (N+1) i)].
__global__ void k_modal_check(const Fields F, int nq, unsigned *flag) {
  const int N = F.N;
  const int nh = (N - 1) * N;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * nh) return;
  const bool hor = t < nh;
  const int r = hor ? t : t - nh;
  size_t f0;
  const size_t stride = (size_t)(N + 1) * N;
  const double *c2, *af, *c2m, *afm, *jc;
  if (hor) {
    f0 = (size_t)(1 + r % (N - 1)) + (size_t)(N + 1) * (r / (N - 1));
    c2 = F.hc2; af = F.haf; c2m = F.hc2m; afm = F.hafm; jc = F.hJC;
  } else {
    f0 = (size_t)(r % N) + (size_t)N * (1 + r / N);
    c2 = F.vc2; af = F.vaf; c2m = F.vc2m; afm = F.vafm; jc = F.vJC;
  }
  bool ok = true, jump = false;
  for (int i = 1; i < nq; ++i) {
    const size_t fi = f0 + stride * i;
    ok = ok && c2[fi] == c2[f0] && af[fi] == af[f0];
    if (F.one_sided) ok = ok && c2m[fi] == c2m[f0] && afm[fi] == afm[f0];
  }
  if (F.one_sided)
    for (int i = 0; i < nq; ++i) jump = jump || jc[f0 + stride * i] != 0.0;
  if (!ok) atomicOr(flag, 1u);
  if (jump) atomicOr(flag, 2u);
}

// The face weights w_i P[i][b] of the projections on the face modes (a kernel parameter)
struct FaceProj {
  double Pw[MAXN][MAXN];
};

// The projections Km[b] = Σ_i w_i P[i][b] K_i of the jump terms K of every face on its nq modes,
// in the face array's layout with mode b in the slot of point b (stride (N+1) N): one thread per
// face of a family of nf faces
__global__ void k_jc_project(const double *jc, int nf, int nq, size_t stride, const FaceProj fp, double *out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  for (int b = 0; b < nq; ++b) {
    double x = 0.0;
    for (int i = 0; i < nq; ++i) x = fma(fp.Pw[i][b], jc[f + stride * i], x);
    out[f + stride * b] = x;
  }
}

// The scratch of the workspace, the kernels' scalars and its stream (the last part of wedg_create)
int create_finish(wedg_ws *ws) {
  const wedg_config *cfg = &ws->cfg;
  const int N = ws->N, E = ws->E, nu = ws->nu, nv = ws->nv, nq = ws->nq, qh = ws->qh;
  const size_t Es = (size_t)E;
  Fields &F = ws->F;
  int rc;
  const size_t nU = (size_t)nu * nu * E, nV = (size_t)nv * nv * E;
  if ((rc = dalloc(ws, &F.tr, (size_t)12 * nq * E)) || (rc = dalloc(ws, &F.G, (size_t)qh * qh * E)) ||
      (rc = dalloc(ws, &F.th, Es)) || (rc = dalloc(ws, &F.de, Es)) || (rc = dalloc(ws, &F.nst, Es)) ||
      (rc = dalloc(ws, &F.nmax, 3)) || (rc = dalloc(ws, &F.nsum, 1)) || (rc = dalloc(ws, &F.err, 1)) ||
      (rc = dalloc(ws, &F.cg_nfail, 1)) ||
      (rc = dalloc(ws, &F.nonfinite, 1)) || (rc = dalloc(ws, &ws->steps_done, 1)) ||
      (rc = dalloc(ws, &ws->d_u, nU)) || (rc = dalloc(ws, &ws->d_v, nV)) || (rc = dalloc(ws, &ws->d_ut, nU)) ||
      (rc = dalloc(ws, &ws->d_vt, nV)) || (rc = dalloc(ws, &ws->su, nU)) || (rc = dalloc(ws, &ws->sv, nV)) ||
      (rc = dalloc(ws, &ws->accu, nU)) || (rc = dalloc(ws, &ws->accv, nV)) || (rc = dalloc(ws, &F.mrhs, nV)) ||
      (rc = dalloc(ws, &F.bins, (size_t)NBIN * E)) || (rc = dalloc(ws, &F.bin_count, (size_t)2 * NBIN)) ||
      (rc = dalloc(ws, &ws->d_flagp, 1)) || (rc = dalloc(ws, &ws->d_flagv, 1))) {
    wedg_destroy(ws);
    return rc;
  }
  {
    const BatchFlagPtrs fp{F.err, F.nsum, F.cg_nfail, F.nonfinite, F.nmax, F.bin_count, ws->steps_done};
    cudaError_t e = cudaMallocHost(&ws->h_flagv, sizeof(BatchFlagVals));
    if (e == cudaSuccess) e = cudaMemcpy(ws->d_flagp, &fp, sizeof fp, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      int r = cuda_fail(ws, e, "wedg_create");
      wedg_destroy(ws);
      return r;
    }
  }
  F.theta = cfg->theta; F.tau = cfg->tau; F.lu = cfg->lambda_u; F.lv = cfg->lambda_v;
  F.omega = cfg->omega;
  const double h = 1.0 / N;
  F.two_h = 2.0 / h;
  F.four_hh = 4.0 / (h * h);
  F.mass_tol = cfg->mass_tol;
  F.Lcheb = std::acosh(1.0 / cfg->mass_tol);
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
  // the dynamic shared-memory opt-in of k_stage on this device (a launch of zero blocks does nothing else)
  cudaError_t ce = ws->L.stage(ws->basis.data(), F, StageIO{}, 0, 0, nullptr);
  if (ce == cudaSuccess) ce = cudaMemset(F.bin_count, 0, 2 * NBIN * sizeof(int));
  if (ce != cudaSuccess) {
    int r = cuda_fail(ws, ce, "wedg_create");
    wedg_destroy(ws);
    return r;
  }
  ce = cudaStreamCreateWithFlags(&ws->own_stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) {
    int r = cuda_fail(ws, ce, "cudaStreamCreate");
    wedg_destroy(ws);
    return r;
  }
  ws->stream = ws->own_stream;
  // traces as modal end sums when every interior face's coefficients are one value along it (after
  // the face arrays' uploads or set-up kernels on any stream)
  const int nface = 2 * (N - 1) * N;
  unsigned flag = cfg->point_traces ? 1u : 0u;
  if (nface > 0 && !flag) {
    unsigned *d = nullptr;
    ce = cudaDeviceSynchronize();
    if (ce == cudaSuccess) ce = cudaMalloc(&d, sizeof(unsigned));
    if (ce == cudaSuccess) ce = cudaMemsetAsync(d, 0, sizeof(unsigned), ws->stream);
    if (ce == cudaSuccess) {
      k_modal_check<<<(nface + 255) / 256, 256, 0, ws->stream>>>(F, nq, d);
      ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&flag, d, sizeof(unsigned), cudaMemcpyDeviceToHost, ws->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ws->stream);
    if (d) cudaFree(d);
    if (ce != cudaSuccess) {
      int r = cuda_fail(ws, ce, "wedg_create");
      wedg_destroy(ws);
      return r;
    }
  }
  ws->modal_ok = (flag & 1u) == 0;
  if (ws->modal_ok && (flag & 2u)) {
    // the jump terms' projections on the face modes
    FaceProj fp{};
    for (int i = 0; i < nq; ++i)
      for (int b = 0; b < nq; ++b) fp.Pw[i][b] = ws->bh.Pw[i][b];
    const size_t nf = (size_t)(N + 1) * N;
    double *hm = nullptr, *vm = nullptr;
    int rc = dalloc(ws, &hm, nf * nq);
    if (!rc) rc = dalloc(ws, &vm, nf * nq);
    if (rc) {
      wedg_destroy(ws);
      return rc;
    }
    k_jc_project<<<(int)((nf + 255) / 256), 256, 0, ws->stream>>>(F.hJC, (int)nf, nq, nf, fp, hm);
    k_jc_project<<<(int)((nf + 255) / 256), 256, 0, ws->stream>>>(F.vJC, (int)nf, nq, nf, fp, vm);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ws->stream);
    if (ce != cudaSuccess) {
      int r = cuda_fail(ws, ce, "wedg_create");
      wedg_destroy(ws);
      return r;
    }
    F.hJCm = hm;
    F.vJCm = vm;
  }
  F.modal = ws->modal_ok ? 1 : 0;
  ws->stats.modal_traces = F.modal;
  ws->stats.fast_path = ws->fast ? 1 : 0;
  ws->stats.device_bytes = (int64_t)ws->bytes;
  cudaDeviceSynchronize();
  return WEDG_OK;
}

}  // namespace


extern "C" {

int wedg_create(const wedg_config *cfg, const wedg_pre *pre, wedg_ws **out) {
  if (!out) return WEDG_ERR_ARGUMENT;
  *out = nullptr;
  if (!cfg || !pre) return WEDG_ERR_ARGUMENT;
  int rc = validate_config(cfg);
  if (rc) return rc;
  const double *need[] = {pre->w, pre->P_u, pre->S_u, pre->Ebl_u, pre->Ebr_u, pre->E1bl_u, pre->E1br_u,
                          pre->P_h_v, pre->W2d_h, pre->Cw, pre->Aw, pre->hc2, pre->haf, pre->hcf, pre->hbf,
                          pre->vc2, pre->vaf, pre->vcf, pre->vbf, pre->hc2m, pre->hafm, pre->vc2m, pre->vafm,
                          pre->hJC, pre->vJC, pre->bcB_sp, pre->bcB_spy, pre->bcT_sp, pre->bcT_spy, pre->bcL_sp,
                          pre->bcL_spx, pre->bcR_sp, pre->bcR_spx, pre->PiSP, pre->PiBSP2, pre->PiCdiv,
                          pre->PiDdiv, pre->src_projE, pre->beta_hq};
  for (const double *p : need)
    if (!p) return WEDG_ERR_ARGUMENT;
  wedg_ws *ws = nullptr;
  if ((rc = create_begin(cfg, pre, &ws))) return rc;
  const int N = ws->N, E = ws->E, nu = ws->nu, nv = ws->nv, nq = ws->nq, qh = ws->qh;
  const size_t Es = (size_t)E;
  BasisHost &bh = ws->bh;

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
  if ((rc = create_launchers(ws, fast))) return rc;

#define UP(dst, vec)                     \
  do {                                   \
    rc = upload(ws, &(dst), vec);        \
    if (rc) { wedg_destroy(ws); return rc; } \
  } while (0)
  Fields &F = ws->F;
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
    } else if ((rc = device_inverses(ws, pre))) {
      return rc;
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
  if ((rc = upload_boundary(ws, pre))) return rc;
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
  F.one_sided = cfg->one_sided ? 1 : 0;
  if ((rc = create_finish(ws))) return rc;
  *out = ws;
  return WEDG_OK;
}

int wedg_create_points(const wedg_config *cfg, const wedg_pre *pre, const wedg_points *pts, char *msg, size_t msg_len,
                       wedg_ws **out) {
  if (msg && msg_len) msg[0] = 0;
  if (!out) return WEDG_ERR_ARGUMENT;
  *out = nullptr;
  auto refuse = [&](int status, const char *why) {
    if (msg && msg_len) snprintf(msg, msg_len, "%s", why);
    return status;
  };
  if (!cfg || !pre || !pts) return refuse(WEDG_ERR_ARGUMENT, "null argument");
  int rc = validate_config(cfg);
  if (rc) return refuse(rc, rc == WEDG_ERR_NO_DEVICE ? "no usable CUDA device" : "invalid configuration");
  const double *need[] = {pre->w, pre->P_u, pre->S_u, pre->Ebl_u, pre->Ebr_u, pre->E1bl_u, pre->E1br_u,
                          pre->P_h_v, pre->W2d_h, pre->bcB_sp, pre->bcB_spy, pre->bcT_sp, pre->bcT_spy,
                          pre->bcL_sp, pre->bcL_spx, pre->bcR_sp, pre->bcR_spx};
  for (const double *p : need)
    if (!p) return refuse(WEDG_ERR_ARGUMENT, "null 1D operator or boundary data");
  const wedg_face_values *fam[6] = {&pts->hc, &pts->ha, &pts->hb, &pts->vc, &pts->va, &pts->vb};
  for (const wedg_face_values *f : fam)
    if (f->at && (!f->lo || !f->hi)) return refuse(WEDG_ERR_ARGUMENT, "null face values");
  if (!cfg->src_on && ((pts->hg0.at && (!pts->hg0.lo || !pts->hg0.hi)) || (pts->vg0.at && (!pts->vg0.lo || !pts->vg0.hi)) ||
                       !pts->cdiv_h || (cfg->mms_on && (!pts->sp_h || !pts->ddiv_h))))
    return refuse(WEDG_ERR_ARGUMENT, "null initial-data or manufactured-solution arrays");
  if (!pts->xloc_h || !pts->yloc_h) return refuse(WEDG_ERR_ARGUMENT, "null high-order points");
  const wedg_cell_table *tabs[3] = {&pts->c_cells, &pts->alpha_cells, &pts->beta_cells};
  for (const wedg_cell_table *t : tabs)
    if (t->values && (t->rows < 1 || t->cols < 1 || !pts->xloc || !pts->yloc))
      return refuse(WEDG_ERR_ARGUMENT, "a cell table needs its sizes and the points xloc, yloc");
  wedg_ws *ws = nullptr;
  if ((rc = create_begin(cfg, pre, &ws))) return refuse(rc, "the quadrature rules are not mirror-symmetric");
  const int N = ws->N, E = ws->E, nv = ws->nv, nq = ws->nq, qh = ws->qh;
  const size_t nE = (size_t)E * nq * nq, nH = (size_t)E * qh * qh, nF = (size_t)nq * (N + 1) * N;
  auto cuda_refuse = [&](cudaError_t e) {
    cuda_fail(ws, e, "wedg_create_points");
    if (msg && msg_len) snprintf(msg, msg_len, "%s", ws->message.c_str());
    wedg_destroy(ws);
    return (int)WEDG_ERR_CUDA;
  };
  // ---- the point arrays on the device, freed when this call returns
  RunBuffers T;
  double *d_c, *d_a, *d_b, *d_w, *d_Ph, *d_Wh, *d_face[6][3], *d_tab[3] = {nullptr, nullptr, nullptr};
  double *d_xq = nullptr, *d_yq = nullptr;
  unsigned long long *d_max;
  double *d_g0[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  double *d_sp = nullptr, *d_cdiv = nullptr, *d_ddiv = nullptr, *d_xh = nullptr, *d_yh = nullptr;
  unsigned *d_flags;
  cudaError_t ce;
  auto put = [&](double **d, const double *h, size_t n) -> cudaError_t {
    cudaError_t e = T.get(d, n);
    if (e == cudaSuccess) e = cudaMemcpy(*d, h, n * sizeof(double), cudaMemcpyHostToDevice);
    return e;
  };
  d_c = d_a = d_b = nullptr;
  if ((pts->c_q && (ce = put(&d_c, pts->c_q, nE)) != cudaSuccess) ||
      (pts->alpha_q && (ce = put(&d_a, pts->alpha_q, nE)) != cudaSuccess) ||
      (pts->beta_h && (ce = put(&d_b, pts->beta_h, nH)) != cudaSuccess) || (ce = put(&d_w, pre->w, nq)) != cudaSuccess ||
      (ce = put(&d_Ph, pre->P_h_v, (size_t)qh * nv)) != cudaSuccess ||
      (ce = put(&d_Wh, pre->W2d_h, (size_t)qh * qh)) != cudaSuccess || (ce = T.get(&d_flags, 1)) != cudaSuccess ||
      (ce = cudaMemset(d_flags, 0, sizeof(unsigned))) != cudaSuccess)
    return cuda_refuse(ce);
  for (int f = 0; f < 6; ++f) {
    const double *src[3] = {fam[f]->at, fam[f]->lo, fam[f]->hi};
    for (int x = 0; x < 3; ++x) {
      d_face[f][x] = nullptr;
      if (src[0] && (ce = put(&d_face[f][x], src[x], nF)) != cudaSuccess) return cuda_refuse(ce);
    }
  }
  if (!cfg->src_on) {
    const wedg_face_values *g[2] = {&pts->hg0, &pts->vg0};
    for (int f = 0; f < 2; ++f) {
      const double *src[3] = {g[f]->at, g[f]->lo, g[f]->hi};
      for (int x = 0; x < 3; ++x)
        if (src[0] && (ce = put(&d_g0[f][x], src[x], nF)) != cudaSuccess) return cuda_refuse(ce);
    }
    if ((ce = put(&d_cdiv, pts->cdiv_h, nH)) != cudaSuccess) return cuda_refuse(ce);
    if (cfg->mms_on &&
        ((ce = put(&d_sp, pts->sp_h, nH)) != cudaSuccess || (ce = put(&d_ddiv, pts->ddiv_h, nH)) != cudaSuccess))
      return cuda_refuse(ce);
  }
  if ((ce = put(&d_xh, pts->xloc_h, (size_t)N * qh)) != cudaSuccess ||
      (ce = put(&d_yh, pts->yloc_h, (size_t)N * qh)) != cudaSuccess ||
      (pts->xloc && (ce = put(&d_xq, pts->xloc, (size_t)N * nq)) != cudaSuccess) ||
      (pts->yloc && (ce = put(&d_yq, pts->yloc, (size_t)N * nq)) != cudaSuccess) ||
      (ce = T.get(&d_max, 1)) != cudaSuccess)
    return cuda_refuse(ce);
  for (int f = 0; f < 3; ++f)
    if (tabs[f]->values && (ce = put(&d_tab[f], tabs[f]->values, (size_t)tabs[f]->rows * tabs[f]->cols)) != cudaSuccess)
      return cuda_refuse(ce);
  const PtsGrid grid{d_xq, d_yq, d_xh, d_yh, N, 1.0 / N};
  const int tb = 128, eb = (E + tb - 1) / tb;
  // ---- constant coefficients per element? (the test wedg_create applies to pre's Cw, Aw)
  unsigned flags = 0;
  const PtsField fc{d_c, pts->c_value, d_c ? nullptr : d_tab[0], tabs[0]->rows, tabs[0]->cols};
  const PtsField fa{d_a, pts->alpha_value, d_a ? nullptr : d_tab[1], tabs[1]->rows, tabs[1]->cols};
  const PtsField fb{d_b, pts->beta_value, d_b ? nullptr : d_tab[2], tabs[2]->rows, tabs[2]->cols};
  k_pts_check<<<eb, tb>>>(fc, fa, grid, d_w, nq, E, d_flags);
  if ((ce = cudaGetLastError()) != cudaSuccess ||
      (ce = cudaMemcpy(&flags, d_flags, sizeof flags, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_refuse(ce);
  const bool fast = !cfg->general_only && !(flags & PTS_NOT_CONSTANT);
  if ((rc = create_launchers(ws, fast))) return refuse(rc, "unsupported degrees");
  Fields &F = ws->F;
  double *c2e = nullptr, *ae = nullptr, *ic2e = nullptr, *Cw = nullptr, *Aw = nullptr;
  if (fast) {
    if (dalloc(ws, &c2e, E) || dalloc(ws, &ae, E) || dalloc(ws, &ic2e, E)) return cuda_refuse(cudaErrorMemoryAllocation);
    F.c2e = c2e; F.ae = ae; F.ic2e = ic2e;
  } else {
    if (dalloc(ws, &Cw, nE) || dalloc(ws, &Aw, nE)) return cuda_refuse(cudaErrorMemoryAllocation);
    F.Cw = Cw; F.Aw = Aw;
  }
  k_pts_elem<<<eb, tb>>>(fc, fa, grid, d_w, nq, E, c2e, ae, ic2e, Cw, Aw);
  if ((ce = cudaGetLastError()) != cudaSuccess) return cuda_refuse(ce);
  if (!fast && (rc = device_inverses(ws, pre))) return refuse(rc, "a stiffness matrix is not positive definite");
  // ---- face arrays, jump terms, one-sided test
  double *fo[2][7];
  for (int h = 0; h < 2; ++h)
    for (int x = 0; x < 7; ++x)
      if (dalloc(ws, &fo[h][x], nF)) return cuda_refuse(cudaErrorMemoryAllocation);
  if ((ce = cudaMemset(d_flags, 0, sizeof(unsigned))) != cudaSuccess) return cuda_refuse(ce);
  // a family: its arrays, or (no arrays) its table with the tolerance term from the device, or its constant
  auto family = [&](int f, int h, PtsFace &out) -> cudaError_t {
    const wedg_face_values *v = fam[3 * h + f];
    out = PtsFace{d_face[3 * h + f][0], d_face[3 * h + f][1], d_face[3 * h + f][2], v->jump_scale, v->value,
                  nullptr, 0, 0};
    if (v->at || !d_tab[f]) return cudaSuccess;
    out.tab = d_tab[f];
    out.m = tabs[f]->rows;
    out.n = tabs[f]->cols;
    unsigned long long bits = 0;
    cudaError_t e = cudaMemset(d_max, 0, sizeof bits);
    if (e == cudaSuccess) {
      k_pts_face_max<<<(int)std::min<size_t>((2 * nF + 255) / 256, 152 * 16), 256>>>(N, nq, grid, out, d_max);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&bits, d_max, sizeof bits, cudaMemcpyDeviceToHost);
    double mx;
    std::memcpy(&mx, &bits, sizeof mx);
    out.s = 1e-8 * mx;        // JUMP_TOL · max over both orientations (src/solver.jl:387)
    return e;
  };
  for (int h = 0; h < 2; ++h) {
    const wedg_face_values &g = h == 0 ? pts->hg0 : pts->vg0;
    PtsFace pc, pa, pb;
    if ((ce = family(0, h, pc)) != cudaSuccess || (ce = family(1, h, pa)) != cudaSuccess ||
        (ce = family(2, h, pb)) != cudaSuccess)
      return cuda_refuse(ce);
    const PtsFace pg{d_g0[h][0], d_g0[h][1], d_g0[h][2], g.jump_scale, cfg->src_on ? 0.0 : g.value, nullptr, 0, 0};
    const PtsFaceOut o{fo[h][0], fo[h][1], fo[h][2], fo[h][3], fo[h][4], fo[h][5], fo[h][6]};
    k_pts_faces<<<(int)std::min<size_t>((nF + 255) / 256, 152 * 16), 256>>>(N, nq, h == 0, grid, pc, pa, pb, pg, o,
                                                                           d_flags);
  }
  if ((ce = cudaGetLastError()) != cudaSuccess ||
      (ce = cudaMemcpy(&flags, d_flags, sizeof flags, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_refuse(ce);
  F.hc2 = fo[0][0]; F.haf = fo[0][1]; F.hcf = fo[0][2]; F.hbf = fo[0][3]; F.hc2m = fo[0][4]; F.hafm = fo[0][5];
  F.hJC = fo[0][6];
  F.vc2 = fo[1][0]; F.vaf = fo[1][1]; F.vcf = fo[1][2]; F.vbf = fo[1][3]; F.vc2m = fo[1][4]; F.vafm = fo[1][5];
  F.vJC = fo[1][6];
  if (cfg->mms_on && (flags & PTS_JUMPS)) {
    wedg_destroy(ws);
    return refuse(WEDG_ERR_ARGUMENT, "mode = :mms needs c and α continuous across the element faces; "
                                     "use :initial_value or :source for coefficients that jump");
  }
  F.one_sided = (flags & (PTS_JUMPS | PTS_JC)) ? 1 : 0;
  if ((rc = upload_boundary(ws, pre))) return refuse(rc, "boundary data");
  // ---- projections and 2β
  auto proj = [&](double **dst, PtsProj p) -> cudaError_t {
    if (dalloc(ws, dst, (size_t)nv * nv * E)) return cudaErrorMemoryAllocation;
    k_pts_proj<<<eb, tb>>>(grid, qh, nv, d_Ph, d_Wh, p, *dst);
    return cudaGetLastError();
  };
  double *pisp = nullptr, *pib = nullptr, *pic = nullptr, *pid = nullptr, *psrc = nullptr, *beta2 = nullptr;
  if (cfg->mms_on) {
    if ((ce = proj(&pisp, PtsProj{0, d_sp, PtsField{}, 0, 0, 0, 0})) != cudaSuccess ||
        (ce = proj(&pib, PtsProj{1, d_sp, fb, 0, 0, 0, 0})) != cudaSuccess ||
        (ce = proj(&pid, PtsProj{0, d_ddiv, PtsField{}, 0, 0, 0, 0})) != cudaSuccess)
      return cuda_refuse(ce);
    F.PiSP = pisp; F.PiBSP2 = pib; F.PiDdiv = pid;
  }
  if (!cfg->src_on) {
    if ((ce = proj(&pic, PtsProj{0, d_cdiv, PtsField{}, 0, 0, 0, 0})) != cudaSuccess)
      return cuda_refuse(ce);
    F.PiCdiv = pic;
  } else {
    if ((ce = proj(&psrc, PtsProj{2, nullptr, PtsField{}, pts->src_amp, pts->src_x0, pts->src_y0, pts->src_r0})) !=
        cudaSuccess)
      return cuda_refuse(ce);
    F.srcP = psrc;
  }
  if (dalloc(ws, &beta2, nH)) return cuda_refuse(cudaErrorMemoryAllocation);
  k_pts_beta2<<<(int)std::min<size_t>((nH + 255) / 256, 152 * 16), 256>>>(grid, qh, fb, beta2);
  if ((ce = cudaGetLastError()) != cudaSuccess || (ce = cudaDeviceSynchronize()) != cudaSuccess) return cuda_refuse(ce);
  F.beta2 = beta2;
  ws->cfg.one_sided = F.one_sided;
  if ((rc = create_finish(ws))) return refuse(rc, "scratch");
  *out = ws;
  return WEDG_OK;
}

int wedg_one_sided(const wedg_ws *ws) { return ws ? ws->F.one_sided : -1; }

int wedg_export(const wedg_ws *ws, const char *name, double *out, size_t count) {
  if (!ws || !name || !out) return WEDG_ERR_ARGUMENT;
  const Fields &F = ws->F;
  const int N = ws->N, E = ws->E, nq = ws->nq, nv = ws->nv, qh = ws->qh;
  const std::string n(name);
  // the device array, the kind of its layout, its size
  const double *src = nullptr;
  int kind = -1;            // 0: h-faces, 1: v-faces, 2: projections, 3: 2β, 4: per element, 5: Cw, Aw, 6: traces
  const struct {
    const char *name;
    const double *p;
    int kind;
  } tab[] = {{"hc2", F.hc2, 0},      {"haf", F.haf, 0},       {"hcf", F.hcf, 0},         {"hbf", F.hbf, 0},
             {"hc2m", F.hc2m, 0},    {"hafm", F.hafm, 0},     {"hJC", F.hJC, 0},         {"vc2", F.vc2, 1},
             {"vaf", F.vaf, 1},      {"vcf", F.vcf, 1},       {"vbf", F.vbf, 1},         {"vc2m", F.vc2m, 1},
             {"vafm", F.vafm, 1},    {"vJC", F.vJC, 1},       {"PiSP", F.PiSP, 2},       {"PiBSP2", F.PiBSP2, 2},
             {"PiCdiv", F.PiCdiv, 2}, {"PiDdiv", F.PiDdiv, 2}, {"src_projE", F.srcP, 2}, {"beta_hq", F.beta2, 3},
             {"c2e", F.c2e, 4},      {"ae", F.ae, 4},         {"Cw", F.Cw, 5},           {"Aw", F.Aw, 5},
             {"tr", F.tr, 6}};
  for (const auto &t : tab)
    if (n == t.name) {
      src = t.p;
      kind = t.kind;
    }
  if (kind < 0 || !src) return WEDG_ERR_ARGUMENT;
  const size_t sizes[7] = {(size_t)nq * (N + 1) * N, (size_t)nq * N * (N + 1), (size_t)nv * nv * E,
                           (size_t)qh * qh * E,      (size_t)E,                 (size_t)nq * nq * E,
                           (size_t)12 * nq * E};
  const size_t len = sizes[kind];
  if (count != len) return WEDG_ERR_DIMENSION;
  std::vector<double> d(len);
  if (cudaMemcpy(d.data(), src, len * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return WEDG_ERR_CUDA;
  const size_t Es = (size_t)E;
  for (size_t t = 0; t < len; ++t) {
    switch (kind) {
      case 6:     // the traces of the last evaluation, in the device layout [((fam 4 + side) nq + i) E + e]
        out[t] = d[t];
        break;
      case 0: {   // [jf + (N+1)(k + N i)] -> (nq, N+1, N)
        const size_t jf = t % (N + 1), k = (t / (N + 1)) % N, i = t / ((size_t)(N + 1) * N);
        out[i + nq * (jf + (size_t)(N + 1) * k)] = d[t];
        break;
      }
      case 1: {   // [j + N (kf + (N+1) i)] -> (nq, N, N+1)
        const size_t j = t % N, kf = (t / N) % (N + 1), i = t / ((size_t)N * (N + 1));
        out[i + nq * (j + (size_t)N * kf)] = d[t];
        break;
      }
      case 2: {   // [l E + e] -> (nv, nv, N, N)
        const size_t e = t % Es, l = t / Es;
        out[l + (size_t)nv * nv * e] = d[t];
        break;
      }
      case 3: {   // 2β [(r + qh s) E + e] -> β (qh, E, qh)
        const size_t e = t % Es, rs = t / Es, r = rs % qh, s_ = rs / qh;
        out[r + qh * (e + Es * s_)] = 0.5 * d[t];
        break;
      }
      case 4:
        out[t] = d[t];
        break;
      default: {  // [(r + nq s) E + e] -> (nq, E, nq)
        const size_t e = t % Es, rs = t / Es, r = rs % nq, s_ = rs / nq;
        out[r + nq * (e + Es * s_)] = d[t];
      }
    }
  }
  return WEDG_OK;
}

void wedg_destroy(wedg_ws *ws) {
  if (!ws) return;
  if (ws->own_stream) cudaStreamSynchronize(ws->own_stream);
  if (ws->stream) cudaStreamSynchronize(ws->stream);
  drain_events(ws);
  for (cudaEvent_t e : ws->ev_pool) cudaEventDestroy(e);
  if (ws->copy_stream) cudaStreamSynchronize(ws->copy_stream);
  for (void *p : ws->allocs) cudaFree(p);
  if (ws->h_flagv) cudaFreeHost(ws->h_flagv);
  if (ws->own_stream) cudaStreamDestroy(ws->own_stream);
  if (ws->copy_stream) cudaStreamDestroy(ws->copy_stream);
  for (cudaEvent_t e : ws->ev_copy)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : ws->ev_chunk)
    if (e) cudaEventDestroy(e);
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
  const bool host = where == WEDG_HOST;
  // with host state: v is copied in on the copy stream beside u on the workspace's stream, and the
  // final u is copied out while the last stage's mass solve runs (Chebyshev)
  const bool u_early = host && nsteps > 0 && ws->cfg.mass_solver != WEDG_CG;
  // with host state and a step to take, the state comes in by ranges of elements on the copy stream
  // and the first stage's k_prep runs on each range as it arrives (k_prep reads only its own
  // element's state)
  const int tp = ws->prep_threads;
  const int nchunk = host && nsteps > 0 && !ws->timing && ws->E >= kCopyChunks * 4 * tp ? kCopyChunks : 0;
  if ((rc = reset_flags(ws))) return rc;
  if (host) {
    if ((rc = copy_stream_ready(ws))) return rc;
    CK(ws, cudaEventRecord(ws->ev_copy[0], ws->stream));           // after the stream's earlier work
    CK(ws, cudaStreamWaitEvent(ws->copy_stream, ws->ev_copy[0], 0));
    du = ws->d_u; dv = ws->d_v;
    if (nchunk) {
      // element ranges of whole k_prep blocks; the state's rows (one per mode) are E doubles apart
      const StageIO S0 = rk4_stage_io(ws, du, dv, 0, t0, dt, nullptr, 0, nullptr, nullptr);
      StageIO Sp = S0;
      Sp.parity = ws->parity;
      const int nb = (ws->E + tp - 1) / tp, per = (nb + nchunk - 1) / nchunk;
      const size_t row = sizeof(double) * ws->E;
      for (int c = 0; c < nchunk; ++c) {
        const int b0 = c * per, b1 = std::min(nb, b0 + per);
        if (b0 >= b1) break;
        const int e0 = b0 * tp, e1 = std::min(ws->E, b1 * tp);
        const size_t w = sizeof(double) * (size_t)(e1 - e0);
        CK(ws, cudaMemcpy2DAsync(ws->d_u + e0, row, u + e0, row, w, (size_t)ws->nu * ws->nu, cudaMemcpyHostToDevice,
                                 ws->copy_stream));
        CK(ws, cudaMemcpy2DAsync(ws->d_v + e0, row, v + e0, row, w, (size_t)ws->nv * ws->nv, cudaMemcpyHostToDevice,
                                 ws->copy_stream));
        CK(ws, cudaEventRecord(ws->ev_chunk[c], ws->copy_stream));
        CK(ws, cudaStreamWaitEvent(ws->stream, ws->ev_chunk[c], 0));
        CK(ws, ws->L.prep(ws->basis.data(), ws->F, Sp, b1 - b0, tp, ws->stream, e0));
        ws->stats.kernel_launches += 1;
      }
    } else {
      CK(ws, cudaMemcpyAsync(ws->d_v, v, bV, cudaMemcpyHostToDevice, ws->copy_stream));
      CK(ws, cudaMemcpyAsync(ws->d_u, u, bU, cudaMemcpyHostToDevice, ws->stream));
      CK(ws, cudaEventRecord(ws->ev_copy[1], ws->copy_stream));
      CK(ws, cudaStreamWaitEvent(ws->stream, ws->ev_copy[1], 0));
    }
  }
  double t = t0;
  for (int64_t it = 0; it < nsteps; ++it) {
    if ((rc = enqueue_rk4(ws, du, dv, t, dt, stop_nonfinite, nullptr, 0, nullptr, nullptr,
                          u_early && it == nsteps - 1 ? ws->ev_copy[0] : nullptr, it == 0 && nchunk > 0)))
      return rc;
    t += dt;
  }
  if (host) {
    if (u_early) {
      CK(ws, cudaStreamWaitEvent(ws->copy_stream, ws->ev_copy[0], 0));
      CK(ws, cudaMemcpyAsync(u, ws->d_u, bU, cudaMemcpyDeviceToHost, ws->copy_stream));
      CK(ws, cudaEventRecord(ws->ev_copy[1], ws->copy_stream));
    } else {
      CK(ws, cudaMemcpyAsync(u, ws->d_u, bU, cudaMemcpyDeviceToHost, ws->stream));
    }
    CK(ws, cudaMemcpyAsync(v, ws->d_v, bV, cudaMemcpyDeviceToHost, ws->stream));
    if (u_early) CK(ws, cudaStreamWaitEvent(ws->stream, ws->ev_copy[1], 0));   // collect's sync covers it
  }
  rc = collect(ws);
  if (steps_done) *steps_done = ws->stats.steps_done;
  if (finite) *finite = ws->stats.finite;
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
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
  // buckets: the same kernels and the same 1D operators
  for (int i = 0; i < n; ++i) {
    wedg_ws *w = b->ws[i];
    const bool cg = w->cfg.mass_solver == WEDG_CG;
    size_t k = 0;
    for (; k < b->buckets.size(); ++k) {
      const BatchBucket &q = b->buckets[k];
      if (q.nu == w->nu && q.nv == w->nv && q.fast == w->fast && q.cg == cg && q.basis == w->basis) break;
    }
    if (k == b->buckets.size()) {
      BatchBucket q;
      q.nu = w->nu; q.nv = w->nv; q.fast = w->fast; q.cg = cg;
      q.L = w->L;
      q.basis = w->basis;
      b->buckets.push_back(q);
    }
    b->buckets[k].ids.push_back(i);
  }
  const size_t per = (size_t)2 * WEDG_BATCH_CHUNK * 4 * 8;    // doubles of one instance's table
  bool ok = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->half_done[0], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->half_done[1], cudaEventDisableTiming) == cudaSuccess &&
            cudaMallocHost(&b->h_tf, sizeof(double) * per * n) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_tf_all, sizeof(double) * per * n) == cudaSuccess &&
       cudaMalloc(&b->d_flagp, sizeof(BatchFlagPtrs) * n) == cudaSuccess &&
       cudaMalloc(&b->d_flagv, sizeof(BatchFlagVals) * n) == cudaSuccess &&
       cudaMallocHost(&b->h_flagv, sizeof(BatchFlagVals) * n) == cudaSuccess;
  for (int i = 0; i < n && ok; ++i) {
    cudaEvent_t e = nullptr;
    b->d_tf.push_back(b->d_tf_all + per * i);
    ok = cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (ok) b->ijoin.push_back(e);
  }
  if (ok) {
    std::vector<BatchFlagPtrs> fp(n);
    for (int i = 0; i < n; ++i) {
      const Fields &F = b->ws[i]->F;
      fp[i] = BatchFlagPtrs{F.err, F.nsum, F.cg_nfail, F.nonfinite, F.nmax, F.bin_count, b->ws[i]->steps_done};
    }
    ok = cudaMemcpy(b->d_flagp, fp.data(), sizeof(BatchFlagPtrs) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  }
  for (BatchBucket &k : b->buckets) {
    if (!ok) break;
    std::stable_sort(k.ids.begin(), k.ids.end(), [&](int x, int y) { return b->ws[x]->E > b->ws[y]->E; });
    std::vector<StepFlags> fl;
    for (int i : k.ids) fl.push_back(StepFlags{b->ws[i]->F.err, b->ws[i]->F.nonfinite, b->ws[i]->steps_done});
    void *p = nullptr, *q = nullptr;
    ok = cudaStreamCreateWithFlags(&k.st, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&k.join, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&k.fork, cudaEventDisableTiming) == cudaSuccess &&
         cudaMalloc(&p, sizeof(StepFlags) * fl.size()) == cudaSuccess &&
         cudaMalloc(&q, sizeof(FinalArgs) * fl.size()) == cudaSuccess;
    if (p) b->dmem.push_back(p);
    if (q) b->dmem.push_back(q);
    if (!ok) break;
    k.d_flags = static_cast<StepFlags *>(p);
    k.d_final = static_cast<FinalArgs *>(q);
    ok = cudaMemcpy(k.d_flags, fl.data(), sizeof(StepFlags) * fl.size(), cudaMemcpyHostToDevice) == cudaSuccess;
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

int wedg_batch_bucket_count(const wedg_batch *b) { return b ? (int)b->buckets.size() : 0; }

int wedg_batch_get_shape(const wedg_batch *b, int bucket, wedg_batch_shape *out) {
  if (!b || !out || bucket < 0 || bucket >= (int)b->buckets.size()) return WEDG_ERR_ARGUMENT;
  const BatchBucket &k = b->buckets[bucket];
  out->qu1 = k.nu;
  out->qv1 = k.nv;
  out->instances = (int32_t)k.ids.size();
  out->fast = k.fast ? 1 : 0;
  out->prep_threads = k.prep_threads;
  out->mass_threads = k.mass_threads;
  out->persist = k.split ? -1 : k.persist;
  return WEDG_OK;
}

int wedg_batch_set_shape(wedg_batch *b, int bucket, int prep_threads, int mass_threads, int persist) {
  if (!b || bucket < 0 || bucket >= (int)b->buckets.size()) return WEDG_ERR_ARGUMENT;
  auto ok = [](int t) { return t >= 32 && t <= CHEB_THREADS && t % 32 == 0; };
  if (!ok(prep_threads) || !ok(mass_threads) || persist < -1 || persist > 8) return WEDG_ERR_ARGUMENT;
  BatchBucket &k = b->buckets[bucket];
  const bool split = persist < 0;
  if (persist < 0) persist = 0;
  if (k.prep_threads != prep_threads || k.mass_threads != mass_threads || k.persist != persist || k.split != split) {
    k.prep_threads = prep_threads;
    k.mass_threads = mass_threads;
    k.persist = persist;
    k.split = split;
    ++b->shape_gen;
  }
  return WEDG_OK;
}

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
  // ---- flags of every instance reset on the batch's stream (after the instance's own work)
  for (int i = 0; i < n; ++i) {
    wedg_ws *w = b->ws[i];
    w->stats.kernel_launches = 0;
    w->parity = 0;
    w->stats.element_stages = 0;
    BK(cudaEventRecord(b->fork, w->stream));
    BK(cudaStreamWaitEvent(b->main, b->fork, 0));
  }
  k_batch_reset<<<n, 128, 0, b->main>>>(b->d_flagp, n);
  BK(cudaGetLastError());
  // ---- the graphs of one and of kBatchGraphSteps steps of every instance, captured again when
  //      their key changed
  bool same = b->exec[0] && b->gstop == (stop_nonfinite ? 1 : 0) && b->gshape == b->shape_gen;
  for (int i = 0; i < n && same; ++i) same = b->gu[i] == u_dev[i] && b->gv[i] == v_dev[i] && b->gdt[i] == dt[i];
  if (!same) {
    for (int g = 0; g < 2; ++g) {
      if (b->exec[g]) { cudaGraphExecDestroy(b->exec[g]); b->exec[g] = nullptr; }
      if (b->graph[g]) { cudaGraphDestroy(b->graph[g]); b->graph[g] = nullptr; }
    }
    int rc = upload_final_args(b, u_dev, v_dev, dt);
    if (rc) return rc;
    b->step_launches.assign(n, 0);
    for (int g = 0; g < 2; ++g) {
      BK(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
      cudaError_t ce = cudaEventRecord(b->fork, b->main);
      for (size_t q = 0; q < b->buckets.size() && ce == cudaSuccess && rc == WEDG_OK; ++q) {
        BatchBucket &k = b->buckets[q];
        ce = cudaStreamWaitEvent(k.st, b->fork, 0);
        if (ce != cudaSuccess) break;
        for (int i : k.ids) b->ws[i]->stats.kernel_launches = 0;
        rc = enqueue_bucket_step(b, k, u_dev, v_dev, nullptr, dt, stop_nonfinite ? 1 : 0, true, 2 * C,
                                 g == 0 ? 1 : kBatchGraphSteps);
        if (g == 0)
          for (int i : k.ids) b->step_launches[i] = b->ws[i]->stats.kernel_launches;
        if (rc == WEDG_OK) ce = cudaEventRecord(k.join, k.st);
        if (ce == cudaSuccess && rc == WEDG_OK) ce = cudaStreamWaitEvent(b->main, k.join, 0);
      }
      cudaGraph_t gr = nullptr;
      const cudaError_t ce2 = cudaStreamEndCapture(b->main, &gr);
      if (rc != WEDG_OK) {
        if (gr) cudaGraphDestroy(gr);
        return rc;
      }
      if (ce != cudaSuccess || ce2 != cudaSuccess) {
        if (gr) cudaGraphDestroy(gr);
        return cuda_err(ce != cudaSuccess ? ce : ce2);
      }
      b->graph[g] = gr;
      BK(cudaGraphInstantiate(&b->exec[g], gr, 0));
    }
    b->gu.assign(u_dev, u_dev + n);
    b->gv.assign(v_dev, v_dev + n);
    b->gdt.assign(dt, dt + n);
    b->gshape = b->shape_gen;
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
    // instance i's rows from h + i chunk to d_tf[i] + half chunk, d_tf[i] = d_tf_all + i per
    BK(cudaMemcpy2DAsync(b->d_tf_all + (size_t)half * chunk, sizeof(double) * 2 * chunk, h, sizeof(double) * chunk,
                         sizeof(double) * cnt * 32, n, cudaMemcpyHostToDevice, b->main));
    BK(cudaEventRecord(b->half_done[half], b->main));
    for (int64_t it = 0; it < cnt;) {
      const bool many = cnt - it >= kBatchGraphSteps;
      BK(cudaGraphLaunch(b->exec[many ? 1 : 0], b->main));
      it += many ? kBatchGraphSteps : 1;
    }
  }
  k_batch_read<<<(n + 127) / 128, 128, 0, b->main>>>(b->d_flagp, n, b->d_flagv);
  BK(cudaGetLastError());
  BK(cudaMemcpyAsync(b->h_flagv, b->d_flagv, sizeof(BatchFlagVals) * n, cudaMemcpyDeviceToHost, b->main));
  BK(cudaStreamSynchronize(b->main));
#undef BK
  int first = WEDG_OK;
  for (int i = 0; i < n; ++i) {
    wedg_ws *w = b->ws[i];
    const BatchFlagVals &f = b->h_flagv[i];
    const int rc = apply_flags(w, f.err, f.cgf, f.nonf, f.nmax, f.done, f.nsum);
    w->stats.kernel_launches = b->step_launches[i] * nsteps;   // the instance's share of the launches run
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
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return cuda_fail(b->ws[0], cudaGetLastError(), "wedg_batch_autotune");
  }
  // steps RK4 steps of bucket k alone from copies of its instances' states, after one untimed step
  // (CUDA events on the bucket's stream)
  auto trial_bucket = [&](BatchBucket &k, double &ms) -> int {
    for (int i : k.ids) {
      wedg_ws *w = b->ws[i];
      const size_t bU = sizeof(double) * w->E * w->nu * w->nu, bV = sizeof(double) * w->E * w->nv * w->nv;
      cudaStream_t own = w->stream;
      w->stream = k.st;
      int rc = reset_flags(w);
      w->stream = own;
      if (rc) return rc;
      cudaError_t e = cudaMemcpyAsync(su[i], u_dev[i], bU, cudaMemcpyDeviceToDevice, k.st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(sv[i], v_dev[i], bV, cudaMemcpyDeviceToDevice, k.st);
      if (e != cudaSuccess) return cuda_fail(w, e, "wedg_batch_autotune");
    }
    int rc = upload_final_args(b, su.data(), sv.data(), dt);
    if (rc) return rc;
    std::vector<double> t(t0, t0 + n);
    if ((rc = enqueue_bucket_step(b, k, su.data(), sv.data(), t.data(), dt, 0, false, 0))) return rc;
    for (int i : k.ids) t[i] += dt[i];
    CK(b->ws[k.ids[0]], cudaEventRecord(e0, k.st));
    for (int64_t it = 0; it < steps; ++it) {
      if ((rc = enqueue_bucket_step(b, k, su.data(), sv.data(), t.data(), dt, 0, false, 0))) return rc;
      for (int i : k.ids) t[i] += dt[i];
    }
    CK(b->ws[k.ids[0]], cudaEventRecord(e1, k.st));
    CK(b->ws[k.ids[0]], cudaEventSynchronize(e1));
    for (int i : k.ids) {
      rc = collect(b->ws[i]);
      if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
    }
    float f = 0;
    CK(b->ws[k.ids[0]], cudaEventElapsedTime(&f, e0, e1));
    ms = f;
    return WEDG_OK;
  };
  // the whole batch's step time (graph replays from copies of the states)
  auto trial_batch = [&](double &ms) -> int {
    for (int i = 0; i < n; ++i) {
      wedg_ws *w = b->ws[i];
      const size_t bU = sizeof(double) * w->E * w->nu * w->nu, bV = sizeof(double) * w->E * w->nv * w->nv;
      cudaError_t e = cudaMemcpyAsync(su[i], u_dev[i], bU, cudaMemcpyDeviceToDevice, w->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(sv[i], v_dev[i], bV, cudaMemcpyDeviceToDevice, w->stream);
      if (e != cudaSuccess) return cuda_fail(w, e, "wedg_batch_autotune");
    }
    int rc = wedg_batch_rk4_steps(b, su.data(), sv.data(), t0, dt, 1, 0, nullptr, nullptr, nullptr);
    if (rc != WEDG_OK && rc != WEDG_WARN_CG_NOT_CONVERGED) return rc;
    // at least two of the larger graphs, so that the call's fixed costs weigh little
    const int64_t ns = std::max<int64_t>(steps, 2 * kBatchGraphSteps);
    const auto c0 = std::chrono::steady_clock::now();
    rc = wedg_batch_rk4_steps(b, su.data(), sv.data(), t1.data(), dt, ns, 0, nullptr, nullptr, nullptr);
    ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - c0).count() / ns;
    return (rc == WEDG_WARN_CG_NOT_CONVERGED) ? WEDG_OK : rc;
  };
  auto median3 = [](double a, double x, double c) { return std::max(std::min(a, x), std::min(std::max(a, x), c)); };
  const int nb = (int)b->buckets.size();
  std::vector<int> def_p(nb), def_m(nb), def_s(nb);
  for (int q = 0; q < nb; ++q) {
    def_p[q] = b->buckets[q].prep_threads;
    def_m[q] = b->buckets[q].mass_threads;
    def_s[q] = b->buckets[q].split ? -1 : b->buckets[q].persist;
  }
  int rc = WEDG_OK;
  // per bucket, alone: one coordinate at a time; a candidate replaces the incumbent only when it is
  // faster in each of kTuneRepeats paired trials and its median is faster by more than 2 %
  for (int q = 0; q < nb && rc == WEDG_OK; ++q) {
    BatchBucket &k = b->buckets[q];
    // the layout first (one launch per kernel over the bucket, or per-instance launches), then the
    // threads per block of k_prep and of the mass solves, then persistent grids
    const int order[3] = {2, 0, 1};
    for (int oc = 0; oc < 3 && rc == WEDG_OK; ++oc) {
      const int c = order[oc];
      for (int x = 0; x < (c == 2 ? 4 : 3) && rc == WEDG_OK; ++x) {
        const int inc[3] = {k.prep_threads, k.mass_threads, k.split ? -1 : k.persist};
        int cand[3] = {inc[0], inc[1], inc[2]};
        cand[c] = c < 2 ? kTuneThreads[x] : x - 1;                  // persist -1 (split), 0, 1, 2
        if (c == 2 && inc[2] < 0 && cand[2] > 0) continue;          // persistence is a merged layout's
        if (cand[c] == inc[c]) continue;
        double ti[kTuneRepeats], tc[kTuneRepeats];
        bool wins = true;
        for (int r = 0; r < kTuneRepeats && rc == WEDG_OK; ++r) {
          wedg_batch_set_shape(b, q, inc[0], inc[1], inc[2]);
          rc = trial_bucket(k, ti[r]);
          if (rc == WEDG_OK) {
            wedg_batch_set_shape(b, q, cand[0], cand[1], cand[2]);
            rc = trial_bucket(k, tc[r]);
          }
          wins = wins && rc == WEDG_OK && tc[r] < ti[r];
        }
        const bool take = rc == WEDG_OK && wins &&
                          median3(tc[0], tc[1], tc[2]) < kTuneGain * median3(ti[0], ti[1], ti[2]);
        const int *keep = take ? cand : inc;
        wedg_batch_set_shape(b, q, keep[0], keep[1], keep[2]);
      }
    }
  }
  // the whole batch: the tuned shapes are kept only if they beat the defaults in paired trials
  double best = 0;
  if (rc == WEDG_OK) {
    std::vector<int> tp(nb), tm(nb), ts(nb);
    for (int q = 0; q < nb; ++q) {
      tp[q] = b->buckets[q].prep_threads;
      tm[q] = b->buckets[q].mass_threads;
      ts[q] = b->buckets[q].split ? -1 : b->buckets[q].persist;
    }
    auto apply = [&](const std::vector<int> &p, const std::vector<int> &m, const std::vector<int> &s_) {
      for (int q = 0; q < nb; ++q) wedg_batch_set_shape(b, q, p[q], m[q], s_[q]);
    };
    double td[kTuneRepeats], tt[kTuneRepeats];
    bool wins = true;
    for (int r = 0; r < kTuneRepeats && rc == WEDG_OK; ++r) {
      apply(def_p, def_m, def_s);
      rc = trial_batch(td[r]);
      if (rc == WEDG_OK) {
        apply(tp, tm, ts);
        rc = trial_batch(tt[r]);
      }
      wins = wins && rc == WEDG_OK && tt[r] < td[r];
    }
    if (rc == WEDG_OK) {
      const double md = median3(td[0], td[1], td[2]), mt = median3(tt[0], tt[1], tt[2]);
      if (wins && mt < kTuneGain * md) {
        apply(tp, tm, ts);
        best = mt;
      } else {
        apply(def_p, def_m, def_s);
        best = md;
      }
    }
  }
  if (rc != WEDG_OK)
    for (int q = 0; q < nb; ++q) wedg_batch_set_shape(b, q, def_p[q], def_m[q], def_s[q]);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != WEDG_OK) return rc;
  if (best_ms) *best_ms = best;
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
  {
    PointTraces point_traces({ws});
    if ((rc = enqueue_rhs_adjoint(ws, du, dv, t, dlu, dlv, dgu, dgv))) return rc;
  }
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
  return adjoint_forward_group({ws}, &u0, &v0, t0, dt, nsteps, every, &uT, &vT, where);
}

int wedg_rk4_adjoint_reverse(wedg_ws *ws, const double *lam_u, const double *lam_v, double *gu, double *gv,
                             double *g_c2, double *g_alpha, double *g_beta, int where) {
  if (!ws) return WEDG_ERR_ARGUMENT;
  return adjoint_reverse_group({ws}, &lam_u, &lam_v, &gu, &gv, &g_c2, &g_alpha, &g_beta, where);
}

int wedg_rk4_adjoint_forward_many(int n, wedg_ws *const *ws, const double *const *u0, const double *const *v0,
                                  double t0, double dt, int64_t nsteps, int64_t every, double *const *uT,
                                  double *const *vT, int where) {
  if (n < 1 || !ws || !u0 || !v0) return WEDG_ERR_ARGUMENT;
  std::vector<wedg_ws *> G(ws, ws + n);
  for (int i = 0; i < n; ++i) {
    if (!G[i]) return WEDG_ERR_ARGUMENT;
    G[i]->stats.kernel_launches = 0;
    G[i]->rk_ready = false;
    if (!u0[i] || !v0[i]) return argument_error(G[i], "null pointer");
    if (!same_kernels(G[0], G[i]))
      return argument_error(G[i], "the workspaces of a group need the same degrees, coefficient kernels and mass solver");
    for (int j = 0; j < i; ++j)
      if (G[j] == G[i]) return argument_error(G[i], "a workspace appears twice in the group");
  }
  std::vector<double *> ou(n, nullptr), ov(n, nullptr);
  for (int i = 0; i < n; ++i) {
    ou[i] = uT ? uT[i] : nullptr;
    ov[i] = vT ? vT[i] : nullptr;
  }
  return adjoint_forward_group(G, u0, v0, t0, dt, nsteps, every, ou.data(), ov.data(), where);
}

int wedg_rk4_adjoint_reverse_many(int n, wedg_ws *const *ws, const double *const *lam_u, const double *const *lam_v,
                                  double *const *gu, double *const *gv, double *const *g_c2, double *const *g_alpha,
                                  double *const *g_beta, int where) {
  if (n < 1 || !ws || !lam_u || !lam_v || !gu || !gv) return WEDG_ERR_ARGUMENT;
  std::vector<wedg_ws *> G(ws, ws + n);
  for (int i = 0; i < n; ++i) {
    if (!G[i]) return WEDG_ERR_ARGUMENT;
    if (!same_kernels(G[0], G[i]))
      return argument_error(G[i], "the workspaces of a group need the same degrees, coefficient kernels and mass solver");
    for (int j = 0; j < i; ++j)
      if (G[j] == G[i]) return argument_error(G[i], "a workspace appears twice in the group");
  }
  std::vector<double *> pc(n, nullptr), pa(n, nullptr), pb(n, nullptr);
  for (int i = 0; i < n; ++i) {
    pc[i] = g_c2 ? g_c2[i] : nullptr;
    pa[i] = g_alpha ? g_alpha[i] : nullptr;
    pb[i] = g_beta ? g_beta[i] : nullptr;
  }
  return adjoint_reverse_group(G, lam_u, lam_v, gu, gv, pc.data(), pa.data(), pb.data(), where);
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
