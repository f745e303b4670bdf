// Device NUTS (diag_e metric, multinomial sampling, adaptation) for many
// chains: one warp per chain, a state machine that runs until the chain needs
// its next gradient, writes the position it needs it at, and yields.  A
// batched gradient over all chains that yielded follows; the next launch
// resumes every chain with its gradient.  Chains never wait for one another,
// so a chain that finishes a short trajectory starts its next transition at
// once (its next gradient shares the batch with other chains' deep trees).
//
// Restated from (paths relative to the stan-dev/stan tree):
//   base_nuts::transition / build_tree   src/stan/mcmc/hmc/nuts/base_nuts.hpp:78-352
//   adapt_diag_e_nuts::transition        src/stan/mcmc/hmc/nuts/adapt_diag_e_nuts.hpp:25-48
//   base_hmc::init_stepsize, sample_stepsize  src/stan/mcmc/hmc/base_hmc.hpp:93-200
//   diag_e_metric (T, dtau_dp, sample_p) src/stan/mcmc/hmc/hamiltonians/diag_e_metric.hpp:20-50
//   expl_leapfrog                        src/stan/mcmc/hmc/integrators/expl_leapfrog.hpp:16-32
//   stepsize_adaptation                  src/stan/mcmc/stepsize_adaptation.hpp:55-73
//   windowed_adaptation, var_adaptation  src/stan/mcmc/windowed_adaptation.hpp:29-110,
//                                        src/stan/mcmc/var_adaptation.hpp:17-46
//   initialize (random inits, retries)   src/stan/services/util/initialize.hpp:68-227
//   generate_transitions (thinning)      src/stan/services/util/generate_transitions.hpp:51-76
//
// The recursion of build_tree becomes iteration over the 2^d leaves of a new
// subtree: after leaf i, the subtrees completed by that leaf are merged bottom
// up (one merge per trailing one bit of i), each merge doing exactly the
// reference's proposal draw, log-sum-exp and three U-turn checks.  An
// unfinished left sibling of depth l waits in stack level l (proposal point,
// momenta at both ends, summed momentum rho, log sum weight).  Uniform draws
// are therefore consumed in the reference's order.  Elementwise updates use
// explicit round-to-nearest operations so they round exactly like the host
// oracle compiled without contraction.
#include <math.h>
#include <stdlib.h>

#include <atomic>

#include "../../include/gbnuts.h"
#include "../../include/gbnuts_draw_stream.h"
#include "gbnuts_internal.h"
#include "loglik_finalize.cuh"
#include "nuts_device.h"
#include "tc_common.cuh"
#include "team.cuh"

namespace gbn {

#define DMUL(a, b) __dmul_rn((a), (b))
#define DADD(a, b) __dadd_rn((a), (b))
#define DSUB(a, b) __dsub_rn((a), (b))
#define DDIV(a, b) __ddiv_rn((a), (b))

static __device__ __forceinline__ double log1p_exp_d(double a) {
  if (a > 0.0) return a + log1p(exp(-a));
  return log1p(exp(a));
}

// stan::math::log_sum_exp (called at base_nuts.hpp:172,265,323-324)
static __device__ __forceinline__ double log_sum_exp_d(double a, double b) {
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  if (a == -inf) return b;
  if (a == inf && b == inf) return inf;
  if (a > b) return a + log1p_exp_d(b - a);
  return b + log1p_exp_d(a - b);
}

struct Ctx {
  const SamplerCfg& cfg;
  double* vecs;
  int c, tid, nth;  // chain; thread index in the chain's team, team size
  Team tm;
  double* dm;  // dense_e: the chain's A, L, M2 (column-major D x D each); null for diag_e
  __device__ double* slot(int s) const {
    return vecs + ((size_t)c * cfg.n_slots + s) * cfg.ld;
  }
};

// The chain's per-level stack in shared memory (one copy per team).  All
// threads hold the same values; entries read and then rewritten by every
// thread are separated by team barriers so none reads another's new value.
struct Stk {
  double* lsw;
  double* V;
  int* slot;
};

// dense_e: out = A v, row i summed over ascending j (dense_e_metric.hpp:38,
// dtau_dp = inv_e_metric_ * p).  Every thread reads all of v: the caller
// synchronises the team after the last write of v.
static __device__ void metric_apply(const Ctx& x, const double* __restrict__ v,
                                    double* __restrict__ out) {
  const int D = x.cfg.D;
  const double* __restrict__ A = x.dm;
  for (int i = x.tid; i < D; i += x.nth) {
    double s = 0.0;
    for (int j = 0; j < D; ++j) s = DADD(s, DMUL(A[(size_t)j * D + i], v[j]));
    out[i] = s;
  }
}

// dense_e: L with A = L L^T from A's lower triangle, column by column; each
// element's dot product summed over ascending k (the reference factors with
// Eigen's llt() where it draws momenta, dense_e_metric.hpp:54-61).
static __device__ void dense_cholesky(const Ctx& x) {
  const int D = x.cfg.D;
  const double* __restrict__ A = x.dm;
  double* __restrict__ L = x.dm + (size_t)D * D;
  for (int e = x.tid; e < D * D; e += x.nth)
    if (e % D < e / D) L[e] = 0.0;  // strict upper part
  for (int j = 0; j < D; ++j) {
    x.tm.sync();
    for (int i = j + x.tid; i < D; i += x.nth) {
      double v = A[(size_t)j * D + i];
      for (int k = 0; k < j; ++k) v = DSUB(v, DMUL(L[(size_t)k * D + i], L[(size_t)k * D + j]));
      L[(size_t)j * D + i] = v;
    }
    x.tm.sync();
    const double d = sqrt(L[(size_t)j * D + j]);
    x.tm.sync();
    for (int i = j + x.tid; i < D; i += x.nth)
      L[(size_t)j * D + i] = i == j ? d : DDIV(L[(size_t)j * D + i], d);
  }
  x.tm.sync();
}

// T(p) = 1/2 p . (invM p)  (diag_e_metric.hpp:20-22, dense_e_metric.hpp:21-23)
static __device__ double kinetic(const Ctx& x, const double* p) {
  if (x.dm) {
    double* t = x.slot(SL_MS0);
    x.tm.sync();
    metric_apply(x, p, t);
    double s = 0.0;
    for (int i = x.tid; i < x.cfg.D; i += x.nth) s += p[i] * t[i];
    return 0.5 * x.tm.sum(s);
  }
  const double* im = x.slot(SL_INVM);
  double s = 0.0;
#pragma unroll 4
  for (int i = x.tid; i < x.cfg.D; i += x.nth) s += p[i] * DMUL(im[i], p[i]);
  return 0.5 * x.tm.sum(s);
}

// Chain c's uniform and normal #n: the counter-based stream, or a scripted
// one (test hook).
static __device__ __forceinline__ double uniform_n(const SamplerCfg& cfg, int c,
                                                   unsigned long long n) {
  if (cfg.script_u)
    return n < (unsigned long long)cfg.script_len ? cfg.script_u[(size_t)c * cfg.script_len + n]
                                                  : __longlong_as_double(0x7ff8000000000000LL);
  return gbds_uniform_at(cfg.seed, cfg.init_chain_id + (unsigned)c, n);
}
static __device__ __forceinline__ double normal_n(const SamplerCfg& cfg, int c,
                                                  unsigned long long n) {
  if (cfg.script_z)
    return n < (unsigned long long)cfg.script_len ? cfg.script_z[(size_t)c * cfg.script_len + n]
                                                  : __longlong_as_double(0x7ff8000000000000LL);
  return gbds_normal_at(cfg.seed, cfg.init_chain_id + (unsigned)c, n);
}

static __device__ __forceinline__ double draw_uniform(const SamplerCfg& cfg, ChainState& st,
                                                      int c) {
  return uniform_n(cfg, c, st.nu++);
}

// The chain's normals #n0 .. #n0 + D - 1: out[i] = z_i, or z_i / sqrt(im[i])
// with im.  One Box-Muller block (two normals, gbds_normal_pair_at) per
// thread; the scripted stream element by element.
static __device__ void draw_normals(const Ctx& x, unsigned long long n0,
                                    const double* __restrict__ im, double* __restrict__ out) {
  const int D = x.cfg.D;
  if (x.cfg.script_z) {
    for (int i = x.tid; i < D; i += x.nth) {
      const double z = normal_n(x.cfg, x.c, n0 + i);
      out[i] = im ? DDIV(z, __dsqrt_rn(im[i])) : z;
    }
    return;
  }
  const unsigned long long b0 = n0 >> 1;
  const unsigned long long nb = ((n0 + (unsigned long long)D - 1) >> 1) - b0 + 1;
  for (unsigned long long j = x.tid; j < nb; j += x.nth) {
    const unsigned long long b = b0 + j;
    double ze, zo;
    gbds_normal_pair_at(x.cfg.seed, x.cfg.init_chain_id + (unsigned)x.c, b, &ze, &zo);
    const long long ie = (long long)(2 * b - n0);  // -1 when n0 is odd and j = 0
    if (ie >= 0) out[ie] = im ? DDIV(ze, __dsqrt_rn(im[ie])) : ze;
    if (ie + 1 < D) out[ie + 1] = im ? DDIV(zo, __dsqrt_rn(im[ie + 1])) : zo;
  }
}

// sample_p (diag_e_metric.hpp:44-50): p_i = n_i / sqrt(invM_i), D normals.
// dense_e (dense_e_metric.hpp:50-61): p = U^{-1} u with A = U^T U, U = L^T,
// solved column by column from the last: p_j = r_j / U_jj, r_i -= U_ij p_j.
// The normals come from slot SL_ZNEXT when drawn ahead (st.z_ready).
static __device__ void sample_p_dense(const Ctx& x, ChainState& st, double* p) {
  const int D = x.cfg.D;
  const double* __restrict__ L = x.dm + (size_t)D * D;
  double* r = x.slot(SL_MS3);
  x.tm.sync();
  if (st.z_ready) {
    const double* z = x.slot(SL_ZNEXT);
    for (int i = x.tid; i < D; i += x.nth) r[i] = z[i];
  } else {
    draw_normals(x, st.nn, nullptr, r);
  }
  st.nn += D;
  st.z_ready = 0;
  for (int j = D - 1; j >= 0; --j) {
    x.tm.sync();
    const double pj = DDIV(r[j], L[(size_t)j * D + j]);
    for (int i = x.tid; i < j; i += x.nth) r[i] = DSUB(r[i], DMUL(L[(size_t)i * D + j], pj));
    if (x.tid == j % x.nth) p[j] = pj;
  }
}

static __device__ void sample_p(const Ctx& x, ChainState& st, double* p) {
  if (x.dm) {
    sample_p_dense(x, st, p);
    return;
  }
  const double* im = x.slot(SL_INVM);
  if (st.z_ready) {
    const double* z = x.slot(SL_ZNEXT);
    for (int i = x.tid; i < x.cfg.D; i += x.nth) p[i] = DDIV(z[i], __dsqrt_rn(im[i]));
  } else {
    draw_normals(x, st.nn, im, p);
  }
  st.nn += x.cfg.D;
  st.z_ready = 0;
}

static __device__ void copy_vec(const Ctx& x, double* __restrict__ dst,
                                const double* __restrict__ src) {
#pragma unroll 4
  for (int i = x.tid; i < x.cfg.D; i += x.nth) dst[i] = src[i];
}

// begin_update_p / end_update_p: p -= (eps/2) g  (expl_leapfrog.hpp:16-28)
static __device__ void half_kick(const Ctx& x, double* __restrict__ p,
                                 const double* __restrict__ g, double half) {
#pragma unroll 4
  for (int i = x.tid; i < x.cfg.D; i += x.nth) p[i] = DSUB(p[i], DMUL(half, g[i]));
}

// update_q: q += eps * invM p, then request the gradient at q.
static __device__ void drift_and_request(const Ctx& x, double* __restrict__ q,
                                         const double* __restrict__ p, double eps,
                                         double* __restrict__ req) {
  if (x.dm) {
    double* t = x.slot(SL_MS0);
    x.tm.sync();
    metric_apply(x, p, t);
    for (int i = x.tid; i < x.cfg.D; i += x.nth) {
      const double v = DADD(q[i], DMUL(eps, t[i]));
      q[i] = v;
      req[i] = v;
    }
    x.tm.sync();
    return;
  }
  const double* __restrict__ im = x.slot(SL_INVM);
#pragma unroll 4
  for (int i = x.tid; i < x.cfg.D; i += x.nth) {
    double v = DADD(q[i], DMUL(eps, DMUL(im[i], p[i])));
    q[i] = v;
    req[i] = v;
  }
}

// The request as tensor-core coefficient words (features 0..127, zeros past
// D), for the chains-on-M gradient kernel.  Reads back the team's own writes.
// f16: fp16 hi / lo words at the chain's scale 2^-e (largest |theta log2 e|
// in [2^13, 2^14)), e in the exponent word.
static __device__ void pack_request_words(const Ctx& x, const double* rq, uint32_t* w,
                                          int f16) {
  x.tm.sync();
  constexpr int kHalf = 64;
  if (f16) {
    float fmax = 0.f;
    for (int k = x.tid; k < x.cfg.D; k += x.nth) fmax = fmaxf(fmax, fabsf(tc::theta_f32(rq[k])));
    fmax = x.tm.max(fmax);
    const int e = tc::theta_exp_f16(fmax);
    const float scale = tc::exp2_int(-e);
    for (int j = x.tid; j < kHalf; j += x.nth) {
      const int k = 2 * j;
      uint32_t wh, wl;
      tc::theta_words_f16(k < x.cfg.D ? tc::theta_f32(rq[k]) : 0.f,
                          k + 1 < x.cfg.D ? tc::theta_f32(rq[k + 1]) : 0.f, scale, wh, wl);
      w[j] = wh;
      w[kHalf + j] = wl;
    }
    if (x.tid == 0) w[tc::kThetaExpWord] = (uint32_t)e;
    return;
  }
  for (int j = x.tid; j < kHalf; j += x.nth) {
    const int k = 2 * j;
    uint32_t wh, wl;
    tc::theta_words(k < x.cfg.D ? rq[k] : 0.0, k + 1 < x.cfg.D ? rq[k + 1] : 0.0, wh, wl);
    w[j] = wh;
    w[kHalf + j] = wl;
  }
}

// constrained output (write_array): exp for the positive parameters.
static __device__ void write_row(const Ctx& x, const ChainState& st, double* row,
                                 double* diag) {
  const SamplerCfg& cfg = x.cfg;
  const double* q = x.slot(SL_SMP_Q);
  if (x.tid == 0) {
    row[0] = -st.V_smp;
    row[1] = st.accept;
    row[2] = st.eps;
    row[3] = st.depth;
    row[4] = st.n_lf;
    row[5] = st.divergent;
    row[6] = st.energy;
  }
  for (int i = x.tid; i < cfg.D; i += x.nth) {
    double v = q[i];
    if (i == cfg.idx_tau || i == cfg.idx_sigma) v = exp(v);
    row[7 + i] = v;
  }
  if (diag) {
    const double* p = x.slot(SL_SMP_P);
    const double* g = x.slot(SL_SMP_G);
    for (int i = x.tid; i < cfg.D; i += x.nth) {
      diag[i] = q[i];
      diag[cfg.D + i] = p[i];
      diag[2 * cfg.D + i] = g[i];
    }
  }
}

// ---------------------------------------------------------------- adaptation
// stepsize_adaptation::learn_stepsize (stepsize_adaptation.hpp:55-71)
static __device__ void learn_stepsize(const SamplerCfg& cfg, ChainState& st, double stat) {
  st.sa_counter += 1.0;
  stat = stat > 1 ? 1 : stat;
  const double eta = 1.0 / (st.sa_counter + cfg.t0);
  st.sa_s_bar = DADD(DMUL(1.0 - eta, st.sa_s_bar), DMUL(eta, cfg.delta - stat));
  // sqrt and pow of the new counter, drawn ahead when sa_pre_ready
  const double sq = st.sa_pre_ready ? st.sa_pre_sqrt : sqrt(st.sa_counter);
  const double x_eta = st.sa_pre_ready ? st.sa_pre_xeta : pow(st.sa_counter, -cfg.kappa);
  st.sa_pre_ready = 0;
  const double xx = st.sa_mu - DMUL(st.sa_s_bar, sq) / cfg.gamma;
  st.sa_x_bar = DADD(DMUL(1.0 - x_eta, st.sa_x_bar), DMUL(x_eta, xx));
  st.nom_eps = exp(xx);
}

// windowed_adaptation (windowed_adaptation.hpp:80-110); unsigned arithmetic.
static __device__ bool adaptation_window(const ChainState& st) {
  return (st.wa_counter >= st.wa_init_buffer) &&
         (st.wa_counter < st.wa_num_warmup - st.wa_term_buffer) &&
         (st.wa_counter != st.wa_num_warmup);
}
static __device__ bool end_adaptation_window(const ChainState& st) {
  return (st.wa_counter == st.wa_next) && (st.wa_counter != st.wa_num_warmup);
}
static __device__ void compute_next_window(ChainState& st) {
  const unsigned last = st.wa_num_warmup - st.wa_term_buffer - 1u;
  if (st.wa_next == last) return;
  st.wa_size *= 2u;
  st.wa_next = st.wa_counter + st.wa_size;
  if (st.wa_next == last) return;
  unsigned boundary = st.wa_next + 2u * st.wa_size;
  if (boundary >= st.wa_num_warmup - st.wa_term_buffer) st.wa_next = last;
}

// var_adaptation::learn_variance (var_adaptation.hpp:17-46) with Welford's
// estimator; returns 1 on a metric update, -1 on overflow.
static __device__ int learn_variance(const Ctx& x, ChainState& st) {
  const int D = x.cfg.D;
  const double* q = x.slot(SL_SMP_Q);
  double* m = x.slot(SL_WM);
  double* m2 = x.slot(SL_WM2);
  double* var = x.slot(SL_INVM);
  if (adaptation_window(st)) {
    st.w_n += 1.0;
    for (int i = x.tid; i < D; i += x.nth) {
      double delta = DSUB(q[i], m[i]);
      m[i] = DADD(m[i], DDIV(delta, st.w_n));
      m2[i] = DADD(m2[i], DMUL(DSUB(q[i], m[i]), delta));
    }
  }
  if (end_adaptation_window(st)) {
    compute_next_window(st);
    const double n = st.w_n;
    const double a = n / (n + 5.0);
    const double b = 1e-3 * (5.0 / (n + 5.0));
    int bad = 0;
    for (int i = x.tid; i < D; i += x.nth) {
      double v = var[i];
      if (n > 1) v = DDIV(m2[i], n - 1.0);
      v = DADD(DMUL(a, v), b);
      var[i] = v;
      if (!isfinite(v)) bad = 1;
      m[i] = 0.0;
      m2[i] = 0.0;
    }
    st.w_n = 0.0;
    st.wa_counter += 1u;
    bad = x.tm.any(bad) ? 1 : 0;
    return bad ? -1 : 1;
  }
  st.wa_counter += 1u;
  return 0;
}

// covar_adaptation::learn_covariance (covar_adaptation.hpp:17-52) with
// Welford's covariance estimator (m += delta / n, M2 += (q - m) delta^T), then
// the new metric's Cholesky factor; returns 1 on a metric update, -1 on
// overflow.
static __device__ int learn_covariance(const Ctx& x, ChainState& st) {
  const int D = x.cfg.D;
  const double* q = x.slot(SL_SMP_Q);
  double* m = x.slot(SL_WM);
  double* dl = x.slot(SL_MS0);
  double* A = x.dm;
  double* M2 = x.dm + 2 * (size_t)D * D;
  if (adaptation_window(st)) {
    st.w_n += 1.0;
    for (int i = x.tid; i < D; i += x.nth) {
      const double delta = DSUB(q[i], m[i]);
      m[i] = DADD(m[i], DDIV(delta, st.w_n));
      dl[i] = delta;
    }
    x.tm.sync();
    for (int e = x.tid; e < D * D; e += x.nth) {
      const int i = e % D, j = e / D;
      M2[e] = DADD(M2[e], DMUL(DSUB(q[i], m[i]), dl[j]));
    }
    x.tm.sync();
  }
  if (end_adaptation_window(st)) {
    compute_next_window(st);
    const double n = st.w_n;
    const double a = n / (n + 5.0);
    const double b = 1e-3 * (5.0 / (n + 5.0));
    int bad = 0;
    for (int e = x.tid; e < D * D; e += x.nth) {
      double v = A[e];
      if (n > 1) v = DDIV(M2[e], n - 1.0);
      v = DADD(DMUL(a, v), (e % D == e / D) ? b : 0.0);
      A[e] = v;
      if (!isfinite(v)) bad = 1;
      M2[e] = 0.0;
    }
    for (int i = x.tid; i < D; i += x.nth) m[i] = 0.0;
    st.w_n = 0.0;
    st.wa_counter += 1u;
    if (x.tm.any(bad)) return -1;
    dense_cholesky(x);
    return 1;
  }
  st.wa_counter += 1u;
  return 0;
}

// The vector pass of an inner merge: rho and the edge momentum of level l,
// its proposal if the final subtree is selected, and the six U-turn dot
// products (partial per thread).  Pointers of the two subtrees never alias.
static __device__ __forceinline__ void merge_level_pass(
    int D, int tid, int nth, double* __restrict__ IQ, double* __restrict__ IP, double* __restrict__ IG,
    const double* __restrict__ IPB, double* __restrict__ IPE, double* __restrict__ IR,
    const double* __restrict__ CQ, const double* __restrict__ CP, const double* __restrict__ CG,
    const double* __restrict__ CPB, const double* __restrict__ CPE,
    const double* __restrict__ CR, const double* __restrict__ im, bool sel_final,
    const double* __restrict__ ps, int ld, double* dd) {
  double d1a = 0, d1b = 0, d2a = 0, d2b = 0, d3a = 0, d3b = 0;
#pragma unroll 2
  for (int i = tid; i < D; i += nth) {
    const double ipb = IPB[i], ipe = IPE[i], ir = IR[i];
    const double cpb = CPB[i], cpe = CPE[i], cr = CR[i];
    // p_sharp = invM p: diag inline, dense precomputed into ps (4 vectors, ld apart)
    const double psb = ps ? ps[i] : DMUL(im[i], ipb);            // p_sharp_beg
    const double pse = ps ? ps[ld + i] : DMUL(im[i], cpe);       // p_sharp_end
    const double psie = ps ? ps[2 * ld + i] : DMUL(im[i], ipe);  // p_sharp_init_end
    const double psfb = ps ? ps[3 * ld + i] : DMUL(im[i], cpb);  // p_sharp_final_beg
    const double rs = DADD(ir, cr);        // rho_init + rho_final
    const double r2 = DADD(ir, cpb);       // rho_init + p_final_beg
    const double r3 = DADD(cr, ipe);       // rho_final + p_init_end
    d1a += pse * rs;
    d1b += psb * rs;
    d2a += psfb * r2;
    d2b += psb * r2;
    d3a += pse * r3;
    d3b += psie * r3;
    IR[i] = rs;
    IPE[i] = cpe;
    if (sel_final) {
      IQ[i] = CQ[i];
      IP[i] = CP[i];
      IG[i] = CG[i];
    }
  }
  dd[0] = d1a;
  dd[1] = d1b;
  dd[2] = d2a;
  dd[3] = d2b;
  dd[4] = d3a;
  dd[5] = d3b;
}

// The vector pass of the top-level merge: trajectory rho and edge momenta,
// the sample if selected, and the six U-turn dot products (partial per thread).
static __device__ __forceinline__ void merge_top_pass(
    int D, int tid, int nth, bool fwd, bool sel, double* __restrict__ RHO, double* __restrict__ PFF,
    double* __restrict__ PFB, double* __restrict__ PBF, double* __restrict__ PBB,
    double* __restrict__ SQ, double* __restrict__ SP, double* __restrict__ SG,
    const double* __restrict__ CQ, const double* __restrict__ CP, const double* __restrict__ CG,
    const double* __restrict__ CPB, const double* __restrict__ CPE,
    const double* __restrict__ CR, const double* __restrict__ im,
    const double* __restrict__ ps, int ld, double* dd) {
  double d1a = 0, d1b = 0, d2a = 0, d2b = 0, d3a = 0, d3b = 0;
#pragma unroll 2
  for (int i = tid; i < D; i += nth) {
    double rho_bck, rho_fwd, p_ff, p_fb, p_bf, p_bb;
    if (fwd) {
      rho_bck = RHO[i];
      rho_fwd = CR[i];
      p_bf = PFF[i];
      p_fb = CPB[i];
      p_ff = CPE[i];
      p_bb = PBB[i];
    } else {
      rho_fwd = RHO[i];
      rho_bck = CR[i];
      p_fb = PBB[i];
      p_bf = CPB[i];
      p_bb = CPE[i];
      p_ff = PFF[i];
    }
    const double rho = DADD(rho_bck, rho_fwd);
    const double ps_ff = ps ? ps[i] : DMUL(im[i], p_ff);
    const double ps_bb = ps ? ps[ld + i] : DMUL(im[i], p_bb);
    const double ps_fb = ps ? ps[2 * ld + i] : DMUL(im[i], p_fb);
    const double ps_bf = ps ? ps[3 * ld + i] : DMUL(im[i], p_bf);
    const double r2 = DADD(rho_bck, p_fb);
    const double r3 = DADD(rho_fwd, p_bf);
    d1a += ps_ff * rho;
    d1b += ps_bb * rho;
    d2a += ps_fb * r2;
    d2b += ps_bb * r2;
    d3a += ps_ff * r3;
    d3b += ps_bf * r3;
    RHO[i] = rho;
    PFF[i] = p_ff;
    PFB[i] = p_fb;
    PBF[i] = p_bf;
    PBB[i] = p_bb;
    if (sel) {
      SQ[i] = CQ[i];
      SP[i] = CP[i];
      SG[i] = CG[i];
    }
  }
  dd[0] = d1a;
  dd[1] = d1b;
  dd[2] = d2a;
  dd[3] = d2b;
  dd[4] = d3a;
  dd[5] = d3b;
}

// ---------------------------------------------------------------- the machine
// Merges the subtree `cur` (the working leaf, or stack level cur_level) into
// stack level l (its left sibling), as build_tree does after its final
// subtree returns (base_nuts.hpp:321-351).  Returns the U-turn verdict.
static __device__ bool merge_into_level(const Ctx& x, ChainState& st, const Stk& sk, int l,
                                        int cur_level, int wq, int wp, int wg, double cur_lsw,
                                        double cur_V) {
  const SamplerCfg& cfg = x.cfg;
  const int pi = sk.slot[l];
  const int base_i = SL_STACK + 6 * pi;
  double* IQ = x.slot(base_i + 0);
  double* IP = x.slot(base_i + 1);
  double* IG = x.slot(base_i + 2);
  double* IPB = x.slot(base_i + 3);
  double* IPE = x.slot(base_i + 4);
  double* IR = x.slot(base_i + 5);
  const double *CQ, *CP, *CG, *CPB, *CPE, *CR;
  if (cur_level < 0) {
    CQ = x.slot(wq);
    CP = x.slot(wp);
    CG = x.slot(wg);
    CPB = CP;
    CPE = CP;
    CR = CP;
  } else {
    const int base_c = SL_STACK + 6 * sk.slot[cur_level];
    CQ = x.slot(base_c + 0);
    CP = x.slot(base_c + 1);
    CG = x.slot(base_c + 2);
    CPB = x.slot(base_c + 3);
    CPE = x.slot(base_c + 4);
    CR = x.slot(base_c + 5);
  }
  const double init_lsw = sk.lsw[l];
  // log-sum-exp and the acceptance probability, on one warp of the team
  const double2 la = x.tm.one2([&]() {
    const double s = log_sum_exp_d(init_lsw, cur_lsw);
    return make_double2(s, cur_lsw > s ? 1.0 : exp(cur_lsw - s));
  });
  const double lsw_sub = la.x;
  bool sel_final;
  if (cur_lsw > lsw_sub) {
    sel_final = true;
  } else {
    sel_final = draw_uniform(cfg, st, x.c) < la.y;
  }
  const double* ps = nullptr;
  if (x.dm) {
    // dense p_sharp of the four edge momenta, before the pass overwrites them
    double* s0 = x.slot(SL_MS0);
    x.tm.sync();
    metric_apply(x, IPB, s0);
    metric_apply(x, CPE, s0 + cfg.ld);
    metric_apply(x, IPE, s0 + 2 * cfg.ld);
    metric_apply(x, CPB, s0 + 3 * cfg.ld);
    x.tm.sync();
    ps = s0;
  }
  double dd[6];
  merge_level_pass(cfg.D, x.tid, x.nth, IQ, IP, IG, IPB, IPE, IR, CQ, CP, CG, CPB, CPE, CR,
                   x.slot(SL_INVM), sel_final, ps, cfg.ld, dd);
  x.tm.sum6(dd);
  const double d1a = dd[0], d1b = dd[1], d2a = dd[2], d2b = dd[3], d3a = dd[4], d3b = dd[5];
  x.tm.sync();
  if (sel_final) sk.V[l] = cur_V;
  sk.lsw[l] = lsw_sub;
  x.tm.sync();
  return (d1a > 0 && d1b > 0) && (d2a > 0 && d2b > 0) && (d3a > 0 && d3b > 0);
}

// Top-level merge of a completed subtree (base_nuts.hpp:157-192).
static __device__ bool merge_top(const Ctx& x, ChainState& st, const Stk& sk, int cur_level,
                                 int wq, int wp, int wg, double cur_lsw, double cur_V) {
  const SamplerCfg& cfg = x.cfg;
  const double *CQ, *CP, *CG, *CPB, *CPE, *CR;
  if (cur_level < 0) {
    CQ = x.slot(wq);
    CP = x.slot(wp);
    CG = x.slot(wg);
    CPB = CP;
    CPE = CP;
    CR = CP;
  } else {
    const int base_c = SL_STACK + 6 * sk.slot[cur_level];
    CQ = x.slot(base_c + 0);
    CP = x.slot(base_c + 1);
    CG = x.slot(base_c + 2);
    CPB = x.slot(base_c + 3);
    CPE = x.slot(base_c + 4);
    CR = x.slot(base_c + 5);
  }
  st.depth += 1;
  // the acceptance probability and the new log-sum-exp, on one warp
  const double lsw_old = st.lsw;
  const double2 al = x.tm.one2([&]() {
    return make_double2(cur_lsw > lsw_old ? 1.0 : exp(cur_lsw - lsw_old),
                        log_sum_exp_d(lsw_old, cur_lsw));
  });
  bool sel;
  if (cur_lsw > st.lsw) {
    sel = true;
  } else {
    sel = draw_uniform(cfg, st, x.c) < al.x;
  }
  st.lsw = al.y;
  double* RHO = x.slot(SL_RHO);
  double* PFF = x.slot(SL_PFF);
  double* PFB = x.slot(SL_PFB);
  double* PBF = x.slot(SL_PBF);
  double* PBB = x.slot(SL_PBB);
  double* SQ = x.slot(SL_SMP_Q);
  double* SP = x.slot(SL_SMP_P);
  double* SG = x.slot(SL_SMP_G);
  const double* im = x.slot(SL_INVM);
  const bool fwd = st.dir > 0;
  const double* ps = nullptr;
  if (x.dm) {
    // dense p_sharp of p_ff, p_bb, p_fb, p_bf as the pass will select them
    double* s0 = x.slot(SL_MS0);
    x.tm.sync();
    metric_apply(x, fwd ? CPE : PFF, s0);
    metric_apply(x, fwd ? PBB : CPE, s0 + cfg.ld);
    metric_apply(x, fwd ? CPB : PBB, s0 + 2 * cfg.ld);
    metric_apply(x, fwd ? PFF : CPB, s0 + 3 * cfg.ld);
    x.tm.sync();
    ps = s0;
  }
  double dd[6];
  merge_top_pass(cfg.D, x.tid, x.nth, fwd, sel, RHO, PFF, PFB, PBF, PBB, SQ, SP, SG, CQ, CP, CG, CPB,
                 CPE, CR, im, ps, cfg.ld, dd);
  if (sel) st.V_smp = cur_V;
  x.tm.sum6(dd);
  const double d1a = dd[0], d1b = dd[1], d2a = dd[2], d2b = dd[3], d3a = dd[4], d3b = dd[5];
  return (d1a > 0 && d1b > 0) && (d2a > 0 && d2b > 0) && (d3a > 0 && d3b > 0);
}

static __device__ void finish_chain(ChainState& st, int status, int* done_count, int tid) {
  st.status = status;
  st.done = 1;
  st.phase = PH_DONE;
  if (tid == 0) atomicAdd(done_count, 1);
}

// One chain's step: runs its state machine from where it yielded to its next
// gradient request (or to the end of its run).  Called by a whole warp.
static __device__ __forceinline__ void nuts_step_chain(const SamplerCfg& cfg, const ModelDesc& m,
                                                       const FitPtrs& f, int c, const Team& tm,
                                                       double* lsw_s, double* V_s, int* slot_s,
                                                       double* cs_s) {
  const int tid = tm.t, nth = tm.n;
  ChainState* __restrict__ states = f.states;
  ChainStack* __restrict__ stacks = f.stacks;
  double* vecs = f.vecs;
  double* __restrict__ req = f.req;
  const PartialsView pv = f.pv;
  int* __restrict__ active = f.active;
  double* __restrict__ draws = f.draws;
  double* __restrict__ diag = f.diag;
  double* __restrict__ init_out = f.init_out;
  const double* __restrict__ inits = f.inits;
  int* __restrict__ done_count = f.done_count;
  const int* __restrict__ abort_flag = f.abort_flag;
  uint32_t* req_tc = f.req_tc ? f.req_tc + (size_t)c * tc::kThetaWords : nullptr;
  ChainState st = states[c];
  if (st.done) {
    if (tid == 0) active[c] = 0;
    return;
  }
  if (tid < MAX_TREE_DEPTH) {
    lsw_s[tid] = stacks[c].lsw[tid];
    slot_s[tid] = stacks[c].slot[tid];
  } else if (tid < 2 * MAX_TREE_DEPTH) {
    V_s[tid - MAX_TREE_DEPTH] = stacks[c].V[tid - MAX_TREE_DEPTH];
  }
  tm.sync();
  const Stk sk{lsw_s, V_s, slot_s};
  Ctx x{cfg, vecs, c, tid, nth, tm,
        f.dense ? f.dense + (size_t)c * 3 * cfg.D * cfg.D : nullptr};
  const int D = cfg.D;
  double* rq = req + (size_t)c * cfg.ld;
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  const double log08 = -0.22314355131420976;  // log(0.8)
  bool yield = false;
  bool light = true;  // no transition or step-size phase in this launch so far
  int guard = 0;
  // The gradient requested at the previous yield, finalised from the split
  // partials into the working point's g slot (g = -grad lp); returns V.
  auto resume = [&](int q_slot, int g_slot) -> double {
    const double lp = finalize_chain(m, x.slot(q_slot), c, cfg.C, pv.P, pv.NP, pv.S, pv.Gz,
                                     x.slot(g_slot), -1.0, 1, 1, tm, cs_s, pv.dyn);
    if (isnan(lp)) return lp;
    if (!isfinite(lp)) return inf;
    return -lp;
  };

  while (!yield && !st.done) {
    if (++guard > 64) {
      finish_chain(st, GBNUTS_CHAIN_STEPSIZE_FAILED, done_count, tid);
      break;
    }
    switch (st.phase) {
      case PH_INIT_DRAW: {
        light = false;
        // initialize.hpp:68-227: user values, zeros, or uniform(-R, R)
        double* q = x.slot(SL_FWD_Q);
        for (int i = tid; i < D; i += nth) {
          double v;
          if (inits)
            v = inits[(size_t)c * D + i];
          else if (cfg.init_radius == 0.0)
            v = 0.0;
          else
            v = DMUL(DSUB(2.0 * uniform_n(cfg, c, st.nu + i), 1.0), cfg.init_radius);
          q[i] = v;
          rq[i] = v;
        }
        if (!inits && cfg.init_radius != 0.0) st.nu += D;
        if (req_tc) pack_request_words(x, rq, req_tc, f.req_tc_f16);
        st.phase = PH_INIT_EVAL;
        yield = true;
        break;
      }
      case PH_INIT_EVAL: {
        light = false;
        st.n_grad += 1;
        const double V0 = resume(SL_FWD_Q, SL_FWD_G);
        double gs = 0.0;
        const double* g0 = x.slot(SL_FWD_G);
        for (int i = tid; i < D; i += nth) gs += g0[i];
        gs = tm.sum(gs);
        if (isfinite(V0) && isfinite(gs)) {
          copy_vec(x, x.slot(SL_SMP_Q), x.slot(SL_FWD_Q));
          copy_vec(x, x.slot(SL_SMP_G), x.slot(SL_FWD_G));
          st.V_smp = V0;
          if (init_out) copy_vec(x, init_out + (size_t)c * D, x.slot(SL_SMP_Q));
          if (f.h_init) {
            // the init values for the host drain (util::initialize writes them
            // to the init writer before the step size search)
            copy_vec(x, f.h_init + (size_t)c * D, x.slot(SL_SMP_Q));
            __threadfence_system();
            tm.sync();
            if (tid == 0) *reinterpret_cast<volatile int*>(f.h_flag + 2 * c) = 1;
          }
          if (cfg.adapt) {
            st.ss_ctx = SS_CTX_START;
            st.phase = PH_SS_BEGIN;
          } else {
            st.phase = PH_AFTER_ITER;
          }
        } else {
          st.init_try += 1;
          const int max_tries = (inits || cfg.init_radius == 0.0) ? 1 : 100;
          if (st.init_try >= max_tries)
            finish_chain(st, GBNUTS_CHAIN_INIT_FAILED, done_count, tid);
          else
            st.phase = PH_INIT_DRAW;
        }
        break;
      }
      case PH_SS_BEGIN: {
        // base_hmc::init_stepsize (base_hmc.hpp:93-105)
        if (st.nom_eps == 0 || st.nom_eps > 1e7 || isnan(st.nom_eps)) {
          st.phase = PH_SS_DONE;
          break;
        }
        st.ss_first = 1;
        st.phase = PH_SS_TRIAL;
        break;
      }
      case PH_SS_TRIAL: {
        light = false;
        // z = z_init; sample_p; H0; evolve(nom_epsilon)  (base_hmc.hpp:107-133)
        double* q = x.slot(SL_FWD_Q);
        double* p = x.slot(SL_FWD_P);
        double* g = x.slot(SL_FWD_G);
        copy_vec(x, q, x.slot(SL_SMP_Q));
        copy_vec(x, g, x.slot(SL_SMP_G));
        st.V_fwd = st.V_smp;
        sample_p(x, st, p);
        tm.sync();
        st.ss_H0 = kinetic(x, p) + st.V_fwd;
        const double e = st.nom_eps;
        half_kick(x, p, g, 0.5 * e);
        drift_and_request(x, q, p, e, rq);
        if (req_tc) pack_request_words(x, rq, req_tc, f.req_tc_f16);
        st.phase = PH_SS_EVAL;
        yield = true;
        break;
      }
      case PH_SS_EVAL: {
        light = false;
        st.n_grad += 1;
        double* p = x.slot(SL_FWD_P);
        double* g = x.slot(SL_FWD_G);
        st.V_fwd = resume(SL_FWD_Q, SL_FWD_G);
        half_kick(x, p, g, 0.5 * st.nom_eps);
        tm.sync();
        double h = kinetic(x, p) + st.V_fwd;
        if (isnan(h)) h = inf;
        const double dH = st.ss_H0 - h;
        if (st.ss_first) {
          st.ss_dir = dH > log08 ? 1 : -1;
          st.ss_first = 0;
          st.phase = PH_SS_TRIAL;
          break;
        }
        if ((st.ss_dir == 1) && !(dH > log08)) {
          st.phase = PH_SS_DONE;
          break;
        }
        if ((st.ss_dir == -1) && !(dH < log08)) {
          st.phase = PH_SS_DONE;
          break;
        }
        st.nom_eps = st.ss_dir == 1 ? 2.0 * st.nom_eps : 0.5 * st.nom_eps;
        if (st.nom_eps > 1e7 || st.nom_eps == 0) {
          finish_chain(st,
                       st.ss_ctx == SS_CTX_START ? GBNUTS_CHAIN_STEPSIZE_INIT_FAILED
                                                 : GBNUTS_CHAIN_STEPSIZE_FAILED,
                       done_count, tid);
          st.ss_fail = st.nom_eps > 1e7 ? 1 : 2;
          break;
        }
        st.phase = PH_SS_TRIAL;
        break;
      }
      case PH_SS_DONE: {
        if (st.ss_ctx == SS_CTX_WINDOW) {
          // adapt_diag_e_nuts.hpp:35-39
          st.sa_mu = log(10 * st.nom_eps);
          st.sa_counter = 0;
          st.sa_pre_ready = 0;
          st.sa_s_bar = 0;
          st.sa_x_bar = 0;
        }
        st.phase = PH_AFTER_ITER;
        break;
      }
      case PH_AFTER_ITER: {
        light = false;
        if (st.adapt_flag && st.iter == cfg.num_warmup) {
          // disengage_adaptation (adapt_diag_e_nuts.hpp:45-48)
          st.adapt_flag = 0;
          st.nom_eps = exp(st.sa_x_bar);
          st.warm_end_ngrad = st.n_grad;
        } else if (!cfg.adapt && st.iter == cfg.num_warmup && st.warm_end_ngrad < 0) {
          st.warm_end_ngrad = st.n_grad;
        }
        if (f.h_adapt && st.iter == cfg.num_warmup) {
          // the adaptation record for the host drain: the step size and the
          // inverse metric the sampling iterations use
          const int M = x.dm ? D * D : D;
          double* rec = f.h_adapt + (size_t)c * (1 + M);
          const double* src = x.dm ? x.dm : x.slot(SL_INVM);
          for (int i = tid; i < M; i += nth) rec[1 + i] = src[i];
          if (tid == 0) rec[0] = st.nom_eps;
          __threadfence_system();
          tm.sync();
          if (tid == 0) *reinterpret_cast<volatile int*>(f.h_flag + 2 * c + 1) = 1;
        }
        if (st.iter >= cfg.num_warmup + cfg.num_samples) {
          finish_chain(st, GBNUTS_CHAIN_OK, done_count, tid);
          break;
        }
        if (abort_flag && *abort_flag) {
          finish_chain(st, GBNUTS_CHAIN_INTERRUPTED, done_count, tid);
          break;
        }
        st.phase = PH_TRANS_BEGIN;
        break;
      }
      case PH_TRANS_BEGIN: {
        light = false;
        // base_nuts::transition (base_nuts.hpp:78-121)
        st.eps = st.nom_eps;
        if (cfg.jitter != 0.0)
          st.eps = DMUL(st.eps,
                        DADD(1.0, DMUL(cfg.jitter, DSUB(2.0 * draw_uniform(cfg, st, c), 1.0))));
        double* SP = x.slot(SL_SMP_P);
        sample_p(x, st, SP);
        tm.sync();
        const double* SQ = x.slot(SL_SMP_Q);
        const double* SG = x.slot(SL_SMP_G);
        double* FQ = x.slot(SL_FWD_Q);
        double* FP = x.slot(SL_FWD_P);
        double* FG = x.slot(SL_FWD_G);
        double* BQ = x.slot(SL_BCK_Q);
        double* BP = x.slot(SL_BCK_P);
        double* BG = x.slot(SL_BCK_G);
        double* PFF = x.slot(SL_PFF);
        double* PFB = x.slot(SL_PFB);
        double* PBF = x.slot(SL_PBF);
        double* PBB = x.slot(SL_PBB);
        double* RHO = x.slot(SL_RHO);
        for (int i = tid; i < D; i += nth) {
          const double q = SQ[i], p = SP[i], g = SG[i];
          FQ[i] = q;
          FP[i] = p;
          FG[i] = g;
          BQ[i] = q;
          BP[i] = p;
          BG[i] = g;
          PFF[i] = p;
          PFB[i] = p;
          PBF[i] = p;
          PBB[i] = p;
          RHO[i] = p;
        }
        st.V_fwd = st.V_smp;
        st.V_bck = st.V_smp;
        st.H0 = kinetic(x, SP) + st.V_smp;
        st.lsw = 0.0;
        st.n_lf = 0;
        st.sum_metro = 0.0;
        st.depth = 0;
        st.divergent = 0;
        st.phase = PH_DOUBLING;
        break;
      }
      case PH_DOUBLING: {
        if (st.depth >= cfg.max_depth) {
          st.phase = PH_TRANS_END;
          break;
        }
        st.dir = draw_uniform(cfg, st, c) > 0.5 ? 1 : -1;
        st.sub_d = st.depth;
        st.leaf = 0;
        tm.sync();
        if (tid < MAX_TREE_DEPTH) sk.slot[tid] = tid;
        tm.sync();
        st.phase = PH_LEAF_BEGIN;
        break;
      }
      case PH_LEAF_BEGIN: {
        const bool fwd = st.dir > 0;
        double* q = x.slot(fwd ? SL_FWD_Q : SL_BCK_Q);
        double* p = x.slot(fwd ? SL_FWD_P : SL_BCK_P);
        const double* g = x.slot(fwd ? SL_FWD_G : SL_BCK_G);
        const double e = st.dir * st.eps;
        half_kick(x, p, g, 0.5 * e);
        drift_and_request(x, q, p, e, rq);
        if (req_tc) pack_request_words(x, rq, req_tc, f.req_tc_f16);
        if (light) {
          // in a short step, draw ahead what the end of the transition needs
          if (!st.z_ready) {
            draw_normals(x, st.nn, nullptr, x.slot(SL_ZNEXT));
            st.z_ready = 1;
          }
          if (st.adapt_flag && !st.sa_pre_ready) {
            const double c1 = st.sa_counter + 1.0;
            st.sa_pre_sqrt = sqrt(c1);
            st.sa_pre_xeta = pow(c1, -cfg.kappa);
            st.sa_pre_ready = 1;
          }
        }
        st.phase = PH_LEAF_EVAL;
        yield = true;
        break;
      }
      case PH_LEAF_EVAL: {
        st.n_grad += 1;
        const bool fwd = st.dir > 0;
        const int wq = fwd ? SL_FWD_Q : SL_BCK_Q;
        const int wp = fwd ? SL_FWD_P : SL_BCK_P;
        const int wg = fwd ? SL_FWD_G : SL_BCK_G;
        double* p = x.slot(wp);
        double* g = x.slot(wg);
        const double V = resume(wq, wg);
        if (fwd)
          st.V_fwd = V;
        else
          st.V_bck = V;
        const double e = st.dir * st.eps;
        half_kick(x, p, g, 0.5 * e);
        tm.sync();
        // leaf of build_tree (base_nuts.hpp:253-281)
        st.n_lf += 1;
        double h = kinetic(x, p) + V;
        if (isnan(h)) h = inf;
        if ((h - st.H0) > 1000.0) st.divergent = 1;
        const double w = st.H0 - h;
        if (w > 0)
          st.sum_metro += 1;
        else
          st.sum_metro += tm.one([&]() { return exp(w); });
        if (st.divergent) {
          st.phase = PH_TRANS_END;
          break;
        }
        const int d = st.sub_d;
        const int i = st.leaf;
        int l = 0;
        int cur_level = -1;
        double cur_lsw = w;
        double cur_V = V;
        bool ok = true;
        while (l < d && ((i >> l) & 1)) {
          tm.sync();
          ok = merge_into_level(x, st, sk, l, cur_level, wq, wp, wg, cur_lsw, cur_V);
          cur_level = l;
          cur_lsw = sk.lsw[l];
          cur_V = sk.V[l];
          ++l;
          if (!ok) break;
        }
        if (!ok) {
          st.phase = PH_TRANS_END;
          break;
        }
        if (l < d) {
          if (cur_level < 0) {
            // push the leaf as the left sibling at level 0
            const int base_i = SL_STACK + 6 * sk.slot[0];
            double* IQ = x.slot(base_i + 0);
            double* IP = x.slot(base_i + 1);
            double* IG = x.slot(base_i + 2);
            double* IPB = x.slot(base_i + 3);
            double* IPE = x.slot(base_i + 4);
            double* IR = x.slot(base_i + 5);
            const double* Q = x.slot(wq);
            for (int k = tid; k < D; k += nth) {
              const double pk = p[k];
              IQ[k] = Q[k];
              IP[k] = pk;
              IG[k] = g[k];
              IPB[k] = pk;
              IPE[k] = pk;
              IR[k] = pk;
            }
            tm.sync();
            sk.lsw[0] = w;
            sk.V[0] = V;
            tm.sync();
          } else {
            // the merged subtree at level l-1 becomes the left sibling at level l
            const int sa = sk.slot[l], sb = sk.slot[l - 1];
            const double la = sk.lsw[l - 1], va = sk.V[l - 1];
            tm.sync();
            sk.slot[l] = sb;
            sk.slot[l - 1] = sa;
            sk.lsw[l] = la;
            sk.V[l] = va;
            tm.sync();
          }
          st.leaf += 1;
          st.phase = PH_LEAF_BEGIN;
          break;
        }
        tm.sync();
        const bool persist = merge_top(x, st, sk, cur_level, wq, wp, wg, cur_lsw, cur_V);
        st.phase = persist ? PH_DOUBLING : PH_TRANS_END;
        break;
      }
      case PH_TRANS_END: {
        // base_nuts.hpp:195-203, then generate_transitions' write and
        // adapt_diag_e_nuts' learning
        light = false;
        tm.sync();
        st.accept = st.sum_metro / (double)st.n_lf;
        st.energy = kinetic(x, x.slot(SL_SMP_P)) + st.V_smp;
        const int m = st.iter;
        bool save;
        if (m < cfg.num_warmup)
          save = cfg.save_warmup && (m % cfg.num_thin) == 0;
        else
          save = ((m - cfg.num_warmup) % cfg.num_thin) == 0;
        if (save && st.rows < cfg.max_rows) {
          double* row = draws + ((size_t)c * cfg.max_rows + st.rows) * cfg.n_cols;
          double* dg = diag ? diag + ((size_t)c * cfg.max_rows + st.rows) * 3 * D : nullptr;
          write_row(x, st, row, dg);
          if (f.h_rows) {
            // the same row into the host drain's array, then the row count
            const size_t ri = (size_t)c * cfg.max_rows + st.rows;
            write_row(x, st, f.h_rows + ri * cfg.n_cols, f.h_diag ? f.h_diag + ri * 3 * D : nullptr);
            __threadfence_system();
            tm.sync();
            if (tid == 0) *reinterpret_cast<volatile int*>(f.h_count + c) = st.rows + 1;
          }
          st.rows += 1;
          if (m < cfg.num_warmup) st.warm_rows += 1;
        }
        st.iter += 1;
        st.phase = PH_AFTER_ITER;
        if (st.adapt_flag) {
          learn_stepsize(cfg, st, st.accept);
          tm.sync();
          const int upd = x.dm ? learn_covariance(x, st) : learn_variance(x, st);
          if (upd < 0) {
            finish_chain(st, GBNUTS_CHAIN_METRIC_OVERFLOW, done_count, tid);
            break;
          }
          if (upd > 0) {
            st.ss_ctx = SS_CTX_WINDOW;
            st.phase = PH_SS_BEGIN;
          }
        }
        break;
      }
      default:
        finish_chain(st, GBNUTS_CHAIN_STEPSIZE_FAILED, done_count, tid);
        break;
    }
    tm.sync();
  }
  tm.sync();
  if (tid < MAX_TREE_DEPTH) {
    stacks[c].lsw[tid] = sk.lsw[tid];
    stacks[c].slot[tid] = sk.slot[tid];
  } else if (tid < 2 * MAX_TREE_DEPTH) {
    stacks[c].V[tid - MAX_TREE_DEPTH] = sk.V[tid - MAX_TREE_DEPTH];
  }
  if (tid == 0) {
    states[c] = st;
    active[c] = (yield && !st.done) ? 1 : 0;
  }
}

// Chains of one or many fits in one launch: team g runs chain chain_map[g].y
// of fit chain_map[g].x.  W = 1: one warp per chain, four chains per CTA;
// W > 1: one chain per CTA of W warps (large dimensions).  A single-fit run
// launches the same kernel with a one-entry table, so a fit's arithmetic is
// the same compiled code alone and in a pool.  Each team first copies its
// fit's descriptor to shared memory.  W = 2 is held to 128 registers, eight
// CTAs per SM: 1216 chains resident at once instead of 608 (1.3% faster per
// step at 1024 chains, D = 101, measured).  W = 8 (D above 1024) is held to
// 128 registers, two CTAs per SM (12% faster per step than W = 4 at 256
// chains, D = 2013, measured).
template <int W>
__global__ void __launch_bounds__(W == 1 ? 128 : 32 * W, W == 2 ? 8 : (W == 8 ? 2 : 1))
    nuts_step_pool_kernel(const PoolFitDev* __restrict__ fits, const int2* __restrict__ chain_map,
                          int total) {
  constexpr int CPB = (W == 1) ? 4 : 1;  // chains per CTA
  __shared__ double sh_lsw[CPB][MAX_TREE_DEPTH];
  __shared__ double sh_V[CPB][MAX_TREE_DEPTH];
  __shared__ int sh_slot[CPB][MAX_TREE_DEPTH];
  __shared__ double sh_cs[CPB][kMaxColSums];
  __shared__ PoolFitDev sh_fit[CPB];
  __shared__ double sh_red[8 * W];
  static_assert(sizeof(PoolFitDev) % 8 == 0, "descriptor copied as 8-byte words");
  const int g = (W == 1) ? (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5)
                         : (int)blockIdx.x;
  const int t = (W == 1) ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
  const int k = (W == 1) ? (int)(threadIdx.x >> 5) : 0;
  if (g >= total) return;  // uniform per team
  const Team tm{t, 32 * W, W, sh_red, 1};
  const int2 fc = chain_map[g];
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(fits + fc.x);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&sh_fit[k]);
  for (int i = t; i < (int)(sizeof(PoolFitDev) / 8); i += 32 * W) dst[i] = src[i];
  tm.sync();
  const PoolFitDev& pf = sh_fit[k];
  nuts_step_chain(pf.cfg, pf.m, pf.f, fc.y, tm, sh_lsw[k], sh_V[k], sh_slot[k], sh_cs[k]);
}

// Sets every chain's state from the configuration (service set-up,
// hmc_nuts_diag_e_adapt.hpp:360-381).
__global__ void nuts_init_kernel(SamplerCfg cfg, ChainState* states, ChainStack* stacks,
                                 double* vecs, const double* inv_metrics, int* active) {
  const int c = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= cfg.C) return;
  for (int s = 0; s < cfg.n_slots; ++s) {
    double* v = vecs + ((size_t)c * cfg.n_slots + s) * cfg.ld;
    for (int i = lane; i < cfg.ld; i += 32)
      v[i] = (s == SL_INVM) ? (inv_metrics ? (i < cfg.D ? inv_metrics[(size_t)c * cfg.D + i] : 1.0)
                                           : 1.0)
                            : 0.0;
  }
  if (lane < MAX_TREE_DEPTH) {
    stacks[c].lsw[lane] = 0.0;
    stacks[c].V[lane] = 0.0;
    stacks[c].slot[lane] = lane;
  }
  if (lane == 0) {
    ChainState st;
    memset(&st, 0, sizeof(st));
    st.phase = PH_INIT_DRAW;
    st.nom_eps = cfg.stepsize;
    st.eps = cfg.stepsize;
    st.sa_mu = log(10 * cfg.stepsize);
    st.adapt_flag = cfg.adapt;
    st.wa_num_warmup = cfg.wa_num_warmup;
    st.wa_init_buffer = cfg.wa_init_buffer;
    st.wa_term_buffer = cfg.wa_term_buffer;
    st.wa_base_window = cfg.wa_base_window;
    st.wa_counter = 0;
    st.wa_size = cfg.wa_size0;
    st.wa_next = cfg.wa_next0;
    st.warm_end_ngrad = -1;
    states[c] = st;
    active[c] = 0;
  }
}

void launch_nuts_init(const SamplerCfg& cfg, ChainState* states, ChainStack* stacks,
                      double* vecs, const double* inv_metrics, int* active, cudaStream_t s) {
  const int threads = 128;
  const int blocks = (int)(((size_t)cfg.C * 32 + threads - 1) / threads);
  nuts_init_kernel<<<blocks, threads, 0, s>>>(cfg, states, stacks, vecs, inv_metrics, active);
}

static std::atomic<int> g_team_warps{0};
void set_team_warps(int w) {
  g_team_warps.store((w == 1 || w == 2 || w == 4 || w == 8) ? w : 0);
}

int team_warps(int D) {
  const int forced = g_team_warps.load();
  if (forced) return forced;
  return D <= 64 ? 1 : (D <= 1024 ? 2 : 8);
}

void launch_nuts_step_pool(const PoolFitDev* fits, const int2* chain_map, int total, int team,
                           cudaStream_t s) {
  if (total <= 0) return;
  if (team == 1) {
    const int threads = 128;
    const int blocks = (int)(((size_t)total * 32 + threads - 1) / threads);
    nuts_step_pool_kernel<1><<<blocks, threads, 0, s>>>(fits, chain_map, total);
  } else if (team == 2) {
    nuts_step_pool_kernel<2><<<total, 64, 0, s>>>(fits, chain_map, total);
  } else if (team == 4) {
    nuts_step_pool_kernel<4><<<total, 128, 0, s>>>(fits, chain_map, total);
  } else {
    nuts_step_pool_kernel<8><<<total, 256, 0, s>>>(fits, chain_map, total);
  }
}

}  // namespace gbn
