// wedg_rhs_noalloc: one right-hand side evaluation that allocates nothing.
//
// Some callers cannot let a library allocate device memory: programs whose GPU
// memory is owned by another runtime's pool allocator (Julia's CUDA.jl or
// PyTorch's caching allocator holding the device), or code that evaluates the
// right-hand side where allocating or freeing device memory is not allowed
// (cudaFree synchronises the whole device). They cannot create a workspace
// (wedg_create allocates the device copy of `pre` and the scratch). This entry
// point needs no workspace: it takes `pre` from host memory, the state and the
// outputs as device pointers, and keeps everything else it needs on the device
// -- the device-layout copy of `pre`, the traces, the Chebyshev data, the mass
// right-hand side and the error word -- in one file-scope static device array of fixed size
// (WEDG_NOALLOC_BYTES). It calls no cudaMalloc, cudaFree or other allocating
// routine, and uses no host heap. The kernels are those of wedg_rhs.
//
// The array is part of the library's device code, so every GPU that loads the
// library holds it until the process exits. Every call shares it and it keeps
// the last call's contents: each call overwrites what it reads and clears the
// error word and counters first. Calls that overlap on the GPU (from two host
// threads, or on two streams) race on the array and must be serialised by the
// caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/wedg.h"
#include "wedg_basis.h"
#include "wedg_dispatch.h"

namespace wedg {
Launchers get_launchers(int nu, int nv, bool fast);   // wedg_api.cu
}

using namespace wedg;

namespace {

constexpr size_t NOALLOC_DOUBLES = WEDG_NOALLOC_BYTES / sizeof(double);

// the scratch of every call of wedg_rhs_noalloc (see the file comment)
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_DOUBLES];

// its device address, looked up once per device with that device current
void *g_scratch_ptr[MAX_DEVICES];
cudaError_t g_setup_err[MAX_DEVICES];
std::once_flag g_setup_once[MAX_DEVICES];

// Reorders a raw copy of one of pre's arrays into the layout the kernels read:
// mode 0: [a + d0 (b + d1 c)] -> [b + d1 (c + d2 a)]   (the first index becomes the slowest)
// mode 1: [a + d0 (b + d1 c)] -> [b + d1 (a + d0 c)]   (Cw, Aw: the element index b first)
// mode 2: as mode 1, doubled                          (β -> 2β, which the kernels read)
__global__ void k_relayout(const double *in, double *out, int d0, int d1, int d2, int mode) {
  const size_t n = (size_t)d0 * d1 * d2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t a = i % d0, bc = i / d0, b = bc % d1, c = bc / d1;
    const size_t o = mode == 0 ? b + (size_t)d1 * (c + (size_t)d2 * a) : b + (size_t)d1 * (a + (size_t)d0 * c);
    out[o] = mode == 2 ? 2.0 * in[i] : in[i];
  }
}

// c² (or α) per element from the raw (nq, E, nq) array of c²W (or αW), and 1/c²
__global__ void k_elem_coef(const double *raw, int nq, int E, double w00, double *val, double *inv) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    const double x = raw[(size_t)nq * e] / w00;
    val[e] = x;
    if (inv) inv[e] = 1.0 / x;
  }
}

int fail(char *msg, size_t len, int status, const char *text) {
  if (msg && len) snprintf(msg, len, "%s", text);
  return status;
}

size_t round_up(size_t n) { return (n + 31) / 32 * 32; }   // 256-byte offsets

}  // namespace

extern "C" int wedg_rhs_noalloc(const wedg_config *cfg, const wedg_pre *pre, const double *u, const double *v,
                                double t, double *ut, double *vt, void *stream, char *msg, size_t msg_len) {
  if (msg && msg_len) msg[0] = 0;
  if (!cfg || !pre || !u || !v || !ut || !vt) return fail(msg, msg_len, WEDG_ERR_ARGUMENT, "null argument");
  const int N = cfg->N, nu = cfg->qu1, nv = cfg->qv1, nq = nu, qh = cfg->q_high;
  if (N < 1 || nu < 2 || nu > MAXN || !(nv == nu || nv == nu - 1) || qh != qhigh(nu, nv) ||
      (cfg->mass_solver != WEDG_CHEBYSHEV && cfg->mass_solver != WEDG_CG))
    return fail(msg, msg_len, WEDG_ERR_ARGUMENT, "invalid configuration");
  for (int s = 0; s < 4; ++s)
    if (cfg->kind[s] < 0 || cfg->kind[s] > 3) return fail(msg, msg_len, WEDG_ERR_ARGUMENT, "invalid boundary kind");
  const size_t E = (size_t)N * N;
  cudaStream_t st = (cudaStream_t)stream;

  // ---- set-up once per device: the device address of the static array
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
    return fail(msg, msg_len, WEDG_ERR_NO_DEVICE, "no usable CUDA device");
  std::call_once(g_setup_once[dev], [dev] {
    g_setup_err[dev] = cudaGetSymbolAddress(&g_scratch_ptr[dev], g_noalloc_scratch);
  });
  if (g_setup_err[dev] != cudaSuccess) {
    if (msg && msg_len)
      snprintf(msg, msg_len, "cudaGetSymbolAddress of the static scratch failed: %s",
               cudaGetErrorString(g_setup_err[dev]));
    return WEDG_ERR_CUDA;
  }
  double *base = static_cast<double *>(g_scratch_ptr[dev]);

  // ---- 1D operators and the constant-coefficient test (host, on the stack)
  BasisHost bh;
  if (const char *why = build_basis(cfg, pre, bh)) return fail(msg, msg_len, WEDG_ERR_ARGUMENT, why);
  const double w00 = bh.w[0] * bh.w[0];
  bool fast = !cfg->general_only;
  for (size_t e = 0; e < E && fast; ++e) {
    const double c2 = pre->Cw[nq * e] / w00, al = pre->Aw[nq * e] / w00;
    for (int s = 0; s < nq && fast; ++s)
      for (int r = 0; r < nq; ++r) {
        const double W = bh.w[r] * bh.w[s];
        const double cw = pre->Cw[r + nq * (e + E * s)], aw = pre->Aw[r + nq * (e + E * s)];
        if (std::fabs(cw - c2 * W) > 1e-14 * std::fabs(cw) || std::fabs(aw - al * W) > 1e-14 * std::fabs(aw) ||
            !(c2 > 0)) {
          fast = false;
          break;
        }
      }
  }
  if (!fast && !pre->Ainv_u)
    return fail(msg, msg_len, WEDG_ERR_ARGUMENT, "Ainv_u is needed: the coefficients are not constant per element");
  const Launchers Lch = get_launchers(nu, nv, fast);
  if (!Lch.prep) return fail(msg, msg_len, WEDG_ERR_ARGUMENT, "unsupported degrees");
  alignas(16) char basis[8192];
  if (Lch.basis_size > sizeof basis) return fail(msg, msg_len, WEDG_ERR_ARGUMENT, "unsupported degrees");
  Lch.pack(bh, basis);

  // ---- layout of the static array (offsets in doubles, 256-byte aligned)
  const size_t nt = (size_t)nu * nu * (nu * nu + 1) / 2;
  const size_t nh = (size_t)nq * (N + 1) * N, nb = (size_t)nq * N, np = (size_t)nv * nv * E;
  size_t off = 0;
  auto take = [&](size_t n) { const size_t o = off; off += round_up(n); return o; };
  const size_t o_flags = take(8);
  const size_t o_c2e = fast ? take(E) : 0, o_ae = fast ? take(E) : 0, o_ic2e = fast ? take(E) : 0;
  const size_t o_cw = fast ? 0 : take((size_t)nq * nq * E), o_aw = fast ? 0 : take((size_t)nq * nq * E);
  const size_t o_ainv = fast ? 0 : take(nt * E);
  size_t o_face[14];
  for (int f = 0; f < 14; ++f) o_face[f] = take(nh);
  size_t o_bnd[8];
  for (int f = 0; f < 8; ++f) o_bnd[f] = take(nb);
  const size_t o_pisp = cfg->mms_on ? take(np) : 0, o_pib = cfg->mms_on ? take(np) : 0;
  const size_t o_pid = cfg->mms_on ? take(np) : 0;
  const size_t o_pic = cfg->src_on ? 0 : take(np), o_src = cfg->src_on ? take(np) : 0;
  const size_t o_beta = take((size_t)qh * qh * E);
  const size_t o_tr = take((size_t)12 * nq * E), o_G = take((size_t)qh * qh * E);
  const size_t o_th = take(E), o_de = take(E), o_nst = take(E);
  const size_t o_mrhs = take((size_t)nv * nv * E);
  const size_t o_bins = take(((size_t)NBIN * E + 1) / 2), o_bcnt = take(NBIN);   // ints, two per double
  size_t raw_max = fast ? (size_t)nq * nq * E : nt * E;
  raw_max = raw_max > (size_t)qh * qh * E ? raw_max : (size_t)qh * qh * E;
  raw_max = raw_max > nh ? raw_max : nh;
  raw_max = raw_max > np ? raw_max : np;
  const size_t o_raw = take(raw_max);
  if (off > NOALLOC_DOUBLES) {
    if (msg && msg_len)
      snprintf(msg, msg_len,
               "mesh too large for wedg_rhs_noalloc: N = %d, q_u + 1 = %d needs %zu bytes of scratch, the static "
               "array holds %zu bytes (WEDG_NOALLOC_BYTES)",
               N, nu, off * sizeof(double), (size_t)WEDG_NOALLOC_BYTES);
    return WEDG_ERR_ARGUMENT;
  }

  // ---- copy pre into the array in the kernels' layouts (a raw copy, then a relayout kernel)
  double *raw = base + o_raw;
  auto relayout = [&](const double *host, size_t count, double *dst, int d0, int d1, int d2, int mode) -> cudaError_t {
    cudaError_t ce = cudaMemcpyAsync(raw, host, count * sizeof(double), cudaMemcpyHostToDevice, st);
    if (ce != cudaSuccess) return ce;
    const int blocks = (int)((count + 255) / 256 < 4096 ? (count + 255) / 256 : 4096);
    k_relayout<<<blocks, 256, 0, st>>>(raw, dst, d0, d1, d2, mode);
    return cudaGetLastError();
  };
  cudaError_t ce = cudaSuccess;
#define RL(...)                                                                                 \
  do {                                                                                          \
    if ((ce = relayout(__VA_ARGS__)) != cudaSuccess) {                                          \
      if (msg && msg_len) snprintf(msg, msg_len, "CUDA error: %s", cudaGetErrorString(ce));     \
      return WEDG_ERR_CUDA;                                                                     \
    }                                                                                           \
  } while (0)
  const int iE = (int)E;
  if (fast) {
    ce = cudaMemcpyAsync(raw, pre->Cw, (size_t)nq * nq * E * sizeof(double), cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) {
      k_elem_coef<<<(iE + 255) / 256, 256, 0, st>>>(raw, nq, iE, w00, base + o_c2e, base + o_ic2e);
      ce = cudaMemcpyAsync(raw, pre->Aw, (size_t)nq * nq * E * sizeof(double), cudaMemcpyHostToDevice, st);
    }
    if (ce == cudaSuccess) {
      k_elem_coef<<<(iE + 255) / 256, 256, 0, st>>>(raw, nq, iE, w00, base + o_ae, nullptr);
      ce = cudaGetLastError();
    }
    if (ce != cudaSuccess) {
      if (msg && msg_len) snprintf(msg, msg_len, "CUDA error: %s", cudaGetErrorString(ce));
      return WEDG_ERR_CUDA;
    }
  } else {
    RL(pre->Cw, (size_t)nq * nq * E, base + o_cw, nq, iE, nq, 1);
    RL(pre->Aw, (size_t)nq * nq * E, base + o_aw, nq, iE, nq, 1);
    RL(pre->Ainv_u, nt * E, base + o_ainv, (int)nt, iE, 1, 0);
  }
  const double *hsrc[7] = {pre->hc2, pre->haf, pre->hcf, pre->hbf, pre->hc2m, pre->hafm, pre->hJC};
  const double *vsrc[7] = {pre->vc2, pre->vaf, pre->vcf, pre->vbf, pre->vc2m, pre->vafm, pre->vJC};
  for (int f = 0; f < 7; ++f) RL(hsrc[f], nh, base + o_face[f], nq, N + 1, N, 0);
  for (int f = 0; f < 7; ++f) RL(vsrc[f], nh, base + o_face[7 + f], nq, N, N + 1, 0);
  const double *bsrc[8] = {pre->bcB_sp, pre->bcT_sp, pre->bcL_sp, pre->bcR_sp,
                           pre->bcB_spy, pre->bcT_spy, pre->bcL_spx, pre->bcR_spx};
  for (int f = 0; f < 8; ++f) RL(bsrc[f], nb, base + o_bnd[f], nq, N, 1, 0);
  if (cfg->mms_on) {
    RL(pre->PiSP, np, base + o_pisp, nv * nv, iE, 1, 0);
    RL(pre->PiBSP2, np, base + o_pib, nv * nv, iE, 1, 0);
    RL(pre->PiDdiv, np, base + o_pid, nv * nv, iE, 1, 0);
  }
  if (!cfg->src_on) RL(pre->PiCdiv, np, base + o_pic, nv * nv, iE, 1, 0);
  if (cfg->src_on) RL(pre->src_projE, np, base + o_src, nv * nv, iE, 1, 0);
  RL(pre->beta_hq, (size_t)qh * qh * E, base + o_beta, qh, iE, qh, 2);
#undef RL

  // ---- the kernels' view of the array
  Fields F;
  std::memset(&F, 0, sizeof F);
  F.N = N;
  F.E = iE;
  if (fast) { F.c2e = base + o_c2e; F.ae = base + o_ae; F.ic2e = base + o_ic2e; }
  else { F.Cw = base + o_cw; F.Aw = base + o_aw; F.Ainv = base + o_ainv; }
  F.hc2 = base + o_face[0]; F.haf = base + o_face[1]; F.hcf = base + o_face[2]; F.hbf = base + o_face[3];
  F.hc2m = base + o_face[4]; F.hafm = base + o_face[5]; F.hJC = base + o_face[6];
  F.vc2 = base + o_face[7]; F.vaf = base + o_face[8]; F.vcf = base + o_face[9]; F.vbf = base + o_face[10];
  F.vc2m = base + o_face[11]; F.vafm = base + o_face[12]; F.vJC = base + o_face[13];
  for (int s = 0; s < 4; ++s) { F.bsp[s] = base + o_bnd[s]; F.bspn[s] = base + o_bnd[4 + s]; }
  if (cfg->mms_on) { F.PiSP = base + o_pisp; F.PiBSP2 = base + o_pib; F.PiDdiv = base + o_pid; }
  if (!cfg->src_on) F.PiCdiv = base + o_pic;
  if (cfg->src_on) F.srcP = base + o_src;
  F.beta2 = base + o_beta;
  F.tr = base + o_tr;
  F.G = base + o_G;
  F.th = base + o_th;
  F.de = base + o_de;
  F.nst = reinterpret_cast<int *>(base + o_nst);
  F.mrhs = base + o_mrhs;
  F.bins = reinterpret_cast<int *>(base + o_bins);
  F.bin_count = reinterpret_cast<int *>(base + o_bcnt);
  double *flags = base + o_flags;   // err (u64), nsum (u64), cg_nfail, nonfinite (u32), nmax (3 ints)
  F.err = reinterpret_cast<unsigned long long *>(flags);
  F.nsum = reinterpret_cast<unsigned long long *>(flags + 1);
  F.nmax = reinterpret_cast<int *>(flags + 5);
  F.cg_nfail = reinterpret_cast<unsigned int *>(flags + 3);
  F.nonfinite = reinterpret_cast<unsigned int *>(flags + 4);
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

  // ---- time factors of src/rhs.jl:509-511 and the source weights
  StageIO S;
  std::memset(&S, 0, sizeof S);
  const double om = cfg->omega;
  S.ct = cfg->mms_on ? std::cos(om * t) : 0.0;
  S.st = cfg->mms_on ? std::sin(om * t) : 0.0;
  if (cfg->src_on && t < cfg->src_Ts) {
    const double sn = std::sin(M_PI * t / cfg->src_Ts);
    S.srct = std::sin(cfg->src_omega * t) * (sn * sn);
  }
  S.cSP = -(om * om) * S.ct;
  S.cB = -2.0 * (om * om * om) * S.st * S.ct;
  S.cC = 1.0 - S.ct;
  S.cD = om * S.st;
  S.xu = u;
  S.xv = v;
  S.mode = OUT_RHS;
  S.ut = ut;
  S.vt = vt;

  // ---- clear what must start at zero (the array keeps the last call's contents), then run
  if ((ce = cudaMemsetAsync(flags, 0, 8 * sizeof(double), st)) != cudaSuccess ||
      (ce = cudaMemsetAsync(F.bin_count, 0, 2 * NBIN * sizeof(int), st)) != cudaSuccess ||
      (ce = cudaMemsetAsync(F.err, 0xFF, sizeof(unsigned long long), st)) != cudaSuccess) {
    if (msg && msg_len) snprintf(msg, msg_len, "CUDA error: %s", cudaGetErrorString(ce));
    return WEDG_ERR_CUDA;
  }
  const int tp = 128, ts = stage_threads(nu, nv, fast);
  unsigned long long err = 0;
  unsigned int cgf = 0;
  if ((ce = Lch.prep(basis, F, S, (iE + tp - 1) / tp, tp, st, 0)) != cudaSuccess ||
      (ce = Lch.stage(basis, F, S, (iE + ts - 1) / ts, ts, st)) != cudaSuccess ||
      (ce = Lch.mass(basis, F, S, 1, CHEB_THREADS, st)) != cudaSuccess ||
      (ce = cudaGetLastError()) != cudaSuccess ||
      (ce = cudaMemcpyAsync(&err, F.err, sizeof err, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(&cgf, F.cg_nfail, sizeof cgf, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (ce = cudaStreamSynchronize(st)) != cudaSuccess) {
    if (msg && msg_len) snprintf(msg, msg_len, "CUDA error: %s", cudaGetErrorString(ce));
    return WEDG_ERR_CUDA;
  }

  // ---- the reference's error semantics and messages (as wedg_rhs)
  if (err != ERR_NONE) {
    const unsigned cls = (unsigned)(err >> ERR_CLASS_SHIFT);
    const long long key = (long long)(err & ((1ull << ERR_CLASS_SHIFT) - 1));
    static const char *kinds[4] = {"absorbing_2beta", "absorbing", "dirichlet", "wall"};
    if (cls == 0) {
      const int s = (int)((key - 1) / (2LL * nq * N));
      const char *kk = cfg->kb[s] == 2.0 ? "2" : "";
      if (msg && msg_len) {
        if (key % 2 == 1)
          snprintf(msg, msg_len, "boundary weight 1 - %sβv_h ≤ 0 at a face point (%s side)", kk, kinds[cfg->kind[s]]);
        else
          snprintf(msg, msg_len, "boundary weight 1 - %sβg ≤ 0 for the boundary data g (%s side)", kk,
                   kinds[cfg->kind[s]]);
      }
      return WEDG_ERR_BOUNDARY_WEIGHT;
    }
    if (msg && msg_len) {
      if (cfg->mass_solver == WEDG_CG)
        snprintf(msg, msg_len, "mass matrix not positive definite on element (%lld, %lld): 1 - 2βv_h ≤ 0",
                 (key - 1) % N + 1, (key - 1) / N + 1);
      else
        snprintf(msg, msg_len, "mass matrix not positive definite on element %lld: 1 - 2βv_h ≤ 0", key);
    }
    return WEDG_ERR_MASS_NOT_PD;
  }
  if (cgf > 0 && cfg->mass_solver == WEDG_CG) {
    if (msg && msg_len)
      snprintf(msg, msg_len, "mass solve: %u element systems did not reach the tolerance %.1e", cgf, cfg->mass_tol);
    return WEDG_WARN_CG_NOT_CONVERGED;
  }
  return WEDG_OK;
}
