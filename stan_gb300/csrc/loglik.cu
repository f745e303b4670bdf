// Batched log density and gradient for C chains (the sampler's
// update_potential_gradient, src/stan/mcmc/hmc/hamiltonians/base_hamiltonian.hpp:61-70,
// for every chain at once).
//
// Every supported family has the form
//     eta_n = base + tau * z[g(n)] + x_n . beta,     lp = sum_n link(eta_n, y_n) + priors
// so one kernel covers all of them:
//   * loglik_partial_kernel: grid (row split s, chain block).  A CTA stages a
//     tile of X rows in shared memory (converted to the compute type), computes
//     eta for CB chains, applies the link (lp term, residual r = dlp/deta),
//     then accumulates X^T r for its chains over all tiles of its row range.
//     Group sums (sum of r over the rows of each group, for d/dz) come from a
//     warp segmented scan over the group-sorted rows, carried across tiles;
//     split boundaries are group aligned so each group sum has one writer.
//   * loglik_finalize_kernel: per chain, sums the split partials in split
//     order (deterministic) and adds priors, Jacobians and the chain rule
//     through tau = exp(u), sigma = exp(u).
// FP64 form: every operation in double.  FP32 form: X.beta, link and X^T r
// in single precision inside a split, partial and final sums in double.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <stdlib.h>
#include <string.h>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"
#include "loglik_finalize.cuh"

namespace gbn {

static constexpr int kThreads = 256;
static constexpr int kMaxPairs = 32;  // (chain, feature) adjoint pairs per thread
// Designs of up to small_k_max<CT>() features take the per-thread row-run
// form (small_k_rows): 16 in the fp32 form; none in the FP64 form, whose
// kernel at 128 registers would spill its FP64 registers; its tiles hold up
// to kSmallRunRows rows per thread run and about kSmallTileBytes of shared
// memory.
template <typename CT>
__host__ __device__ constexpr int small_k_max() {
  return sizeof(CT) == 8 ? 0 : 16;
}
template <typename CT>
__host__ __device__ inline bool use_small_k(int K) {
  return small_k_max<CT>() > 0 && K >= 1 && K <= small_k_max<CT>();
}
static constexpr int kSmallRunRows = 64;
static constexpr size_t kSmallTileBytes = 64 * 1024;

int chains_per_block(int K) {
  if (K <= 512) return 16;
  if (K <= 1024) return 8;
  if (K <= 2048) return 4;
  return 0;
}

int block_chains(int K, int C) {
  const int by_c = C <= 4 ? 4 : (C <= 8 ? 8 : 16);
  return std::min(chains_per_block(K), by_c);
}

// X element in the compute type, converted once (fp32 X into the fp32 form
// is a plain copy: no pass through double on GB300's FP64 pipe).
template <typename CT, typename XT>
__device__ __forceinline__ CT x_to(XT v) {
  return (CT)v;
}
template <>
__device__ __forceinline__ float x_to<float, uint16_t>(uint16_t v) {
  return __uint_as_float(((unsigned)v) << 16);
}
template <>
__device__ __forceinline__ double x_to<double, uint16_t>(uint16_t v) {
  return (double)__uint_as_float(((unsigned)v) << 16);
}

template <typename CT>
__device__ __forceinline__ void apply_link(int link, CT eta, CT y, CT inv_s2, CT& term,
                                           CT& resid, CT& sq) {
  if (link == LINK_LOGIT) {
    CT e = exp(-fabs(eta));
    CT sp = (eta > CT(0) ? eta : CT(0)) + log1p(e);
    term = y * eta - sp;
    CT sig = eta >= CT(0) ? CT(1) / (CT(1) + e) : e / (CT(1) + e);
    resid = y - sig;
    sq = CT(0);
  } else if (link == LINK_POISSON_LOG) {
    CT mu = exp(eta);
    term = y * eta - mu;
    resid = y - mu;
    sq = CT(0);
  } else {
    CT e = y - eta;
    term = CT(-0.5) * e * e * inv_s2;
    resid = e * inv_s2;
    sq = e * e;
  }
}

// Shared memory of the partial kernel: theta [CB][K + 1], then the tile's
// rows (small-K form: [RB][KS], KS = K rounded up to 16-byte loads; otherwise
// [RB][K + 1] and the residuals [RB][CB]), y, group.
template <typename CT>
__host__ __device__ inline int small_row_stride(int K) {
  constexpr int VW = 16 / sizeof(CT);
  return (K + VW - 1) / VW * VW;
}
template <typename CT>
__host__ __device__ inline size_t partial_smem_bytes(int CB, int K, int RB) {
  const int KP = K + 1;
  if (use_small_k<CT>(K))
    return sizeof(CT) * ((size_t)CB * KP + (size_t)RB * small_row_stride<CT>(K) + RB) +
           sizeof(int) * (size_t)RB;
  return sizeof(CT) * ((size_t)CB * KP + (size_t)RB * KP + (size_t)RB * CB + RB) +
         sizeof(int) * (size_t)RB;
}

// Designs of up to small_k_max<CT>() features (the hierarchical models'
// group-level predictors): each thread owns one chain and a contiguous run of
// RR <= RB / RPT rows of every tile.  Theta, the K adjoint sums and the z of
// the current group stay in registers (z is re-read and converted only when
// the group changes); a row's features are 16-byte loads from shared memory,
// and eta, the link and the adjoint update X^T r run in one pass over the row.
// Group sums: a run's segments are summed in row order; a segment inside a run
// is complete and written at once, and the first and last segments of the
// runs are joined by one thread per chain in run order, carried across tiles.
// Every sum's order depends on the split's rows only (deterministic).
// Shared memory: th_s [CB][K + 1], then the tile's rows [RB][KS] (KS = K
// rounded up to whole 16-byte loads), y, group (partial_smem_bytes).
template <typename XT, typename CT, int CB>
__device__ __forceinline__ void small_k_rows(
    const ModelDesc& m, const double* __restrict__ Q, int ldq, int C, const CT* th_s,
    const CT* base_s, const CT* tau_s, const CT* invs2_s, const int* act_s,
    double (*red_s)[4], int RB, long long row_begin, long long row_end, double* __restrict__ P,
    int NP, double* __restrict__ Gz, int s, int c0, double& lp_d, double& base_d,
    double& tau_d, double& sq_d) {
  constexpr int VW = 16 / sizeof(CT);   // elements per 16-byte load
  constexpr int RPT = kThreads / CB;    // runs (threads) per chain
  const int K = m.K, KP = K + 1;
  const int KS = (K + VW - 1) / VW * VW;
  // rows per run: at most RB / RPT, and the split's rows in tiles of equal
  // size, so every run of every tile has rows (a short split or a short
  // last tile would otherwise leave most runs idle)
  const long long n_split = row_end - row_begin;
  const long long cap = (long long)(RB / RPT) * RPT;
  const long long n_tiles = (n_split + cap - 1) / cap;
  const int RR = n_tiles > 0 ? (int)((n_split + n_tiles * RPT - 1) / (n_tiles * RPT)) : 1;
  const int RBe = RR * RPT;  // rows per tile (<= RB)
  const int dr = kThreads / K, dk = kThreads - (kThreads / K) * K;
  const int tid = threadIdx.x, my_c = tid % CB, my_rl = tid / CB;
  CT* x_s = const_cast<CT*>(th_s) + (size_t)CB * KP;  // [RB][KS]
  CT* y_s = x_s + (size_t)RB * KS;
  int* g_s = reinterpret_cast<int*>(y_s + RB);
  const XT* __restrict__ X = static_cast<const XT*>(m.X);
  const bool has_z = m.off_z >= 0;
  const bool cact = act_s[my_c] != 0;
  struct RunEnds {  // one run's group segments at its two ends (red_s: 32 bytes a thread)
    int fkey, lkey;
    CT fsum, lsum;
  };
  static_assert(sizeof(RunEnds) <= 4 * sizeof(double), "run ends fit a red_s row");
  const int cg = c0 + my_c;
  const double* thq = Q + (size_t)(cact ? cg : 0) * ldq;

  constexpr int SK = small_k_max<CT>() > 0 ? small_k_max<CT>() : 1;
  CT th[SK], acc[SK];
#pragma unroll
  for (int k = 0; k < SK; ++k) {
    th[k] = k < K ? th_s[my_c * KP + k] : CT(0);
    acc[k] = CT(0);
  }
  // feature columns K .. KS-1 stay zero
  for (int idx = tid; idx < RB * (KS - K); idx += kThreads) {
    const int r = idx / (KS - K);
    x_s[r * KS + K + (idx - r * (KS - K))] = CT(0);
  }
  const CT base = base_s[my_c], tau = tau_s[my_c], invs2 = invs2_s[my_c];
  int zkey = -1;
  CT zc = CT(0);
  int carry_key = -1;  // the open group segment (thread my_rl == 0 of each chain)
  CT carry_val = CT(0);
  auto put_gz = [&](int key, CT v) { Gz[(size_t)cg * m.J + key] = (double)v; };

  for (long long r0 = row_begin; r0 < row_end; r0 += RBe) {
    const int nrows = (int)min((long long)RBe, row_end - r0);
    __syncthreads();
    // the tile's rows are contiguous in X: element idx = r K + k, stepped
    // by kThreads = dr K + dk without a division per element
    const XT* xt = X + (size_t)r0 * K;
    {
      int r = tid / K, k = tid - (tid / K) * K;
      for (int idx = tid; idx < nrows * K; idx += kThreads) {
        x_s[r * KS + k] = x_to<CT, XT>(xt[idx]);
        r += dr;
        k += dk;
        if (k >= K) {
          k -= K;
          ++r;
        }
      }
    }
    for (int idx = tid; idx < RBe; idx += kThreads) {
      y_s[idx] = idx < nrows ? (CT)m.y[r0 + idx] : CT(0);
      g_s[idx] = (has_z && idx < nrows) ? m.group[r0 + idx] : -1;
    }
    __syncthreads();

    CT lp_t = 0, base_t = 0, tau_t = 0, sq_t = 0;
    int fkey = -2, ckey = -2;  // first closed segment's group, current segment's
    CT fsum = CT(0), cur = CT(0);
    const int rb0 = my_rl * RR;
    if (cact) {
      for (int j = 0; j < RR; ++j) {
        const int r = rb0 + j;
        if (r >= nrows) break;
        CT xr[SK];
#pragma unroll
        for (int k = 0; k < SK; k += VW) {
          if (k < KS) {
            if (VW == 4) {
              const float4 v = *reinterpret_cast<const float4*>(x_s + r * KS + k);
              xr[k] = v.x;
              xr[k + 1] = v.y;
              xr[k + 2] = v.z;
              xr[k + 3] = v.w;
            } else {
              const double2 v = *reinterpret_cast<const double2*>(x_s + r * KS + k);
              xr[k] = v.x;
              xr[k + 1] = v.y;
            }
          } else {
#pragma unroll
            for (int u = 0; u < VW; ++u) xr[k + u] = CT(0);
          }
        }
        CT dotv = CT(0);
#pragma unroll
        for (int k = 0; k < SK; ++k) dotv = fma(xr[k], th[k], dotv);
        CT eta = base + dotv;
        const int g = g_s[r];
        if (has_z) {
          if (g != zkey) {
            zkey = g;
            zc = (CT)thq[m.off_z + g];
          }
          eta += tau * zc;
        }
        CT term, resid, sq;
        apply_link<CT>(m.link, eta, y_s[r], invs2, term, resid, sq);
        lp_t += term;
        base_t += resid;
        tau_t += resid * zc;
        sq_t += sq;
#pragma unroll
        for (int k = 0; k < SK; ++k) acc[k] = fma(xr[k], resid, acc[k]);
        if (has_z) {
          if (g != ckey) {
            if (ckey >= 0) {
              if (fkey == -2) {
                fkey = ckey;
                fsum = cur;
              } else {
                put_gz(ckey, cur);  // a segment inside the run
              }
            }
            ckey = g;
            cur = CT(0);
          }
          cur += resid;
        }
      }
    }
    lp_d += (double)lp_t;
    base_d += (double)base_t;
    tau_d += (double)tau_t;
    sq_d += (double)sq_t;
    if (has_z) {
      // the run's first closed segment (or -2: one segment) and its last one
      RunEnds* ends = reinterpret_cast<RunEnds*>(red_s);
      ends[tid] = RunEnds{fkey, ckey, fsum, cur};
      __syncthreads();
      if (my_rl == 0 && cact) {
        for (int rl = 0; rl < RPT; ++rl) {
          const RunEnds e = ends[rl * CB + my_c];
          const int fk = e.fkey, lk = e.lkey;
          if (lk < 0) continue;  // no rows
          const CT fs = e.fsum, ls = e.lsum;
          if (fk >= 0) {
            // two or more segments: the first one ends inside this run
            if (fk == carry_key) {
              carry_val += fs;
            } else {
              if (carry_key >= 0) put_gz(carry_key, carry_val);
              carry_val = fs;
            }
            put_gz(fk, carry_val);
            carry_key = lk;
            carry_val = ls;
          } else if (lk == carry_key) {
            carry_val += ls;
          } else {
            if (carry_key >= 0) put_gz(carry_key, carry_val);
            carry_key = lk;
            carry_val = ls;
          }
        }
      }
    }
  }
  if (has_z && my_rl == 0 && cact && carry_key >= 0) put_gz(carry_key, carry_val);

  // X^T r: the runs' sums of each (chain, feature) added in run order
  __syncthreads();
  CT* red = x_s;  // [RPT][CB][K], fits in the tile's rows (RB KS >= RPT CB K)
#pragma unroll
  for (int k = 0; k < SK; ++k)
    if (k < K) red[(size_t)tid * K + k] = acc[k];
  __syncthreads();
  for (int p = tid; p < CB * K; p += kThreads) {
    const int c = p / K, k = p - c * K;
    if (!act_s[c]) continue;
    double a = 0;
    for (int rl = 0; rl < RPT; ++rl) a += (double)red[(size_t)(rl * CB + c) * K + k];
    P[((size_t)s * C + c0 + c) * NP + 4 + k] = a;
  }
}

// One CTA's work: split s of the rows, chain block cb (CB chains), RB rows per
// shared-memory tile.
template <typename XT, typename CT, int CB>
__device__ __forceinline__ void loglik_partial_body(
    const ModelDesc& m, const double* __restrict__ Q, int ldq, int C,
    const int* __restrict__ active, const long long* __restrict__ split_rows, int RB,
    double* __restrict__ P, int NP, double* __restrict__ Gz, int s, int cb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = m.K;
  const int KP = K + 1;
  CT* th_s = reinterpret_cast<CT*>(smem_raw);  // [CB][KP]
  CT* x_s = th_s + (size_t)CB * KP;            // [RB][KP]
  CT* r_s = x_s + (size_t)RB * KP;             // [RB][CB]
  CT* y_s = r_s + (size_t)RB * CB;             // [RB]
  int* g_s = reinterpret_cast<int*>(y_s + RB);  // [RB]
  __shared__ CT base_s[CB], tau_s[CB], invs2_s[CB];
  __shared__ int act_s[CB];
  __shared__ double red_s[kThreads][4];

  const int tid = threadIdx.x;
  const int c0 = cb * CB;
  const XT* __restrict__ X = static_cast<const XT*>(m.X);

  for (int idx = tid; idx < CB * K; idx += kThreads) {
    int c = idx / K, k = idx - c * K;
    int cg = c0 + c;
    th_s[c * KP + k] = (cg < C) ? (CT)Q[(size_t)cg * ldq + m.off_beta + k] : CT(0);
  }
  if (tid < CB) {
    int cg = c0 + tid;
    int act = (cg < C) && (active == nullptr || active[cg] != 0);
    act_s[tid] = act;
    const double* th = Q + (size_t)(act ? cg : 0) * ldq;
    base_s[tid] = (act && m.has_base) ? (CT)th[0] : CT(0);
    tau_s[tid] = (act && m.idx_tau >= 0) ? (CT)exp(th[m.idx_tau]) : CT(0);
    double sig = (act && m.idx_sigma >= 0) ? exp(th[m.idx_sigma]) : 1.0;
    invs2_s[tid] = (CT)(1.0 / (sig * sig));
  }
  int any = (tid < CB) ? act_s[tid] : 0;
  if (!__syncthreads_or(any)) return;

  const long long row_begin = split_rows[s], row_end = split_rows[s + 1];
  constexpr int RPT = kThreads / CB;  // row lanes per pass
  const int my_c = tid % CB, my_rl = tid / CB;
  const int warp = tid >> 5, lane = tid & 31;
  const bool has_z = m.off_z >= 0;
  double lp_d = 0, base_d = 0, tau_d = 0, sq_d = 0;
  if (use_small_k<CT>(K)) {  // RB >= kThreads, whole runs of rows (choose_rb)
    small_k_rows<XT, CT, CB>(m, Q, ldq, C, th_s, base_s, tau_s, invs2_s, act_s, red_s, RB,
                             row_begin, row_end, P, NP, Gz, s, c0, lp_d, base_d, tau_d,
                             sq_d);
  } else {
    CT acc[kMaxPairs];
#pragma unroll
    for (int j = 0; j < kMaxPairs; ++j) acc[j] = CT(0);
    // segmented-scan carry for the group sums, per (warp, chain slot)
    constexpr int kChainsPerWarp = (CB + 7) / 8;
    int carry_key[kChainsPerWarp];
    CT carry_val[kChainsPerWarp];
#pragma unroll
    for (int i = 0; i < kChainsPerWarp; ++i) {
      carry_key[i] = -1;
      carry_val[i] = CT(0);
    }

    for (long long r0 = row_begin; r0 < row_end; r0 += RB) {
      const int nrows = (int)min((long long)RB, row_end - r0);
      __syncthreads();
      const XT* xt = X + (size_t)r0 * K;
      for (int idx = tid; idx < nrows * K; idx += kThreads) {
        int r = idx / K, k = idx - r * K;
        x_s[r * KP + k] = x_to<CT, XT>(xt[idx]);
      }
      for (int idx = tid; idx < RB; idx += kThreads) {
        y_s[idx] = idx < nrows ? (CT)m.y[r0 + idx] : CT(0);
        g_s[idx] = (has_z && idx < nrows) ? m.group[r0 + idx] : -1;
      }
      __syncthreads();

      // forward: eta, link, per-chain scalar sums
      {
        CT lp_t = 0, base_t = 0, tau_t = 0, sq_t = 0;
        const bool cact = act_s[my_c] != 0;
        const CT* tc = th_s + my_c * KP;
        const double* thq = Q + (size_t)(c0 + my_c) * ldq;
        for (int r = my_rl; r < RB; r += RPT) {
          CT resid = CT(0);
          if (cact && r < nrows) {
            const CT* xr = x_s + r * KP;
            CT dotv = CT(0);
            for (int k = 0; k < K; ++k) dotv = fma(xr[k], tc[k], dotv);
            CT eta = base_s[my_c] + dotv;
            CT zg = CT(0);
            if (has_z) {
              zg = (CT)thq[m.off_z + g_s[r]];
              eta += tau_s[my_c] * zg;
            }
            CT term, sq;
            apply_link<CT>(m.link, eta, y_s[r], invs2_s[my_c], term, resid, sq);
            lp_t += term;
            base_t += resid;
            tau_t += resid * zg;
            sq_t += sq;
          }
          r_s[r * CB + my_c] = resid;
        }
        lp_d += (double)lp_t;
        base_d += (double)base_t;
        tau_d += (double)tau_t;
        sq_d += (double)sq_t;
      }
      __syncthreads();

      // adjoint: X^T r for (chain, feature) pairs
#pragma unroll
      for (int j = 0; j < kMaxPairs; ++j) {
        int p = tid + kThreads * j;
        if (p < CB * K) {
          int c = p / K, k = p - c * K;
          CT a = CT(0);
          for (int r = 0; r < nrows; ++r) a = fma(x_s[r * KP + k], r_s[r * CB + c], a);
          acc[j] += a;
        }
      }

      // group sums: warp w handles chain slots w, w + 8, ...
      if (has_z) {
#pragma unroll
        for (int i = 0; i < kChainsPerWarp; ++i) {
          const int c = warp + 8 * i;
          if (c < CB && act_s[c]) {
            const int cg = c0 + c;
            for (int rb = 0; rb < nrows; rb += 32) {
              const int r = rb + lane;
              int key = r < nrows ? g_s[r] : -2 - lane;
              CT val = r < nrows ? r_s[r * CB + c] : CT(0);
#pragma unroll
              for (int off = 1; off < 32; off <<= 1) {
                CT v = __shfl_up_sync(0xffffffffu, val, off);
                int kk = __shfl_up_sync(0xffffffffu, key, off);
                if (lane >= off && kk == key) val += v;
              }
              int next_key = __shfl_down_sync(0xffffffffu, key, 1);
              bool seg_end = (lane == 31) || (next_key != key);
              // the first segment of the chunk continues the carried one
              int first_key = __shfl_sync(0xffffffffu, key, 0);
              if (key == first_key && key == carry_key[i]) val += carry_val[i];
              int last_key = __shfl_sync(0xffffffffu, key, 31);
              CT last_val = __shfl_sync(0xffffffffu, val, 31);
              if (seg_end && r < nrows && lane != 31) Gz[(size_t)cg * m.J + key] = (double)val;
              // the chunk's last segment may continue into the next chunk
              if (last_key >= 0) {
                if (carry_key[i] >= 0 && carry_key[i] != first_key && lane == 0) {
                  // carried segment ended exactly at the previous chunk boundary
                  Gz[(size_t)cg * m.J + carry_key[i]] = (double)carry_val[i];
                }
                carry_key[i] = last_key;
                carry_val[i] = last_val;
              } else {
                // partial chunk ending the tile: last valid lane closes its segment
                // (it was written above unless it is lane 31, impossible here)
                if (carry_key[i] >= 0 && carry_key[i] != first_key && lane == 0)
                  Gz[(size_t)cg * m.J + carry_key[i]] = (double)carry_val[i];
                carry_key[i] = -1;
                carry_val[i] = CT(0);
              }
            }
          }
        }
      }
    }

    // flush open group segments
    if (has_z && lane == 0) {
#pragma unroll
      for (int i = 0; i < kChainsPerWarp; ++i) {
        const int c = warp + 8 * i;
        if (c < CB && act_s[c] && carry_key[i] >= 0)
          Gz[(size_t)(c0 + c) * m.J + carry_key[i]] = (double)carry_val[i];
      }
    }

#pragma unroll
    for (int j = 0; j < kMaxPairs; ++j) {
      int p = tid + kThreads * j;
      if (p < CB * K) {
        int c = p / K, k = p - c * K;
        if (act_s[c]) P[((size_t)s * C + c0 + c) * NP + 4 + k] = (double)acc[j];
      }
    }
  }
  red_s[tid][0] = lp_d;
  red_s[tid][1] = base_d;
  red_s[tid][2] = tau_d;
  red_s[tid][3] = sq_d;
  __syncthreads();
  if (tid < CB && act_s[tid]) {
    double v[4] = {0, 0, 0, 0};
    for (int rl = 0; rl < RPT; ++rl)
      for (int q = 0; q < 4; ++q) v[q] += red_s[rl * CB + tid][q];
    double* dst = P + ((size_t)s * C + c0 + tid) * NP;
    for (int q = 0; q < 4; ++q) dst[q] = v[q];
  }
}

template <typename XT, typename CT, int CB>
__global__ void __launch_bounds__(kThreads)
    loglik_partial_kernel(ModelDesc m, const double* __restrict__ Q, int ldq, int C,
                          const int* __restrict__ active,
                          const long long* __restrict__ split_rows, int RB,
                          double* __restrict__ P, int NP, double* __restrict__ Gz) {
  loglik_partial_body<XT, CT, CB>(m, Q, ldq, C, active, split_rows, RB, P, NP, Gz, blockIdx.x,
                                  blockIdx.y);
}

// Many fits in one launch: CTA b runs work item items[b] (fit, split, chain
// block, tile rows), each fit with its own data and partial buffers.
template <typename XT, typename CT, int CB>
__global__ void __launch_bounds__(kThreads)
    loglik_partial_pool_kernel(const PoolGradFit* __restrict__ fits,
                               const PoolWorkItem* __restrict__ items) {
  const PoolWorkItem it = items[blockIdx.x];
  const PoolGradFit& f = fits[it.fit];
  loglik_partial_body<XT, CT, CB>(f.m, f.Q, f.ldq, f.C, f.active, f.split_rows, it.rb, f.P,
                                  f.NP, f.Gz, it.split, it.chain_block);
}

// Per chain (one warp): split sums + priors + Jacobians -> lp, grad.
__global__ void __launch_bounds__(128)
    loglik_finalize_kernel(ModelDesc m, const double* __restrict__ Q, int ldq, int C,
                           const int* __restrict__ active, const double* __restrict__ P,
                           int NP, int S, const double* __restrict__ Gz,
                           double* __restrict__ lp_out, double* __restrict__ grad, int ldg,
                           int propto, int jacobian, const int* __restrict__ dyn) {
  __shared__ double sh_cs[4][kMaxColSums];
  const int c = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= C) return;  // uniform per warp
  if (active && !active[c]) return;
  const Team tm{lane, 32, 1, nullptr};
  const double lp = finalize_chain(m, Q + (size_t)c * ldq, c, C, P, NP, S, Gz,
                                   grad + (size_t)c * ldg, 1.0, propto, jacobian, tm,
                                   sh_cs[threadIdx.x >> 5], dyn);
  if (lane == 0) lp_out[c] = lp;
}

// ------------------------------------------------------------------ host side
template <typename XT, typename CT, int CB>
static int set_smem_attr(size_t bytes) {
  return ensure_smem(loglik_partial_kernel<XT, CT, CB>, bytes);
}

static constexpr size_t kSmemBudget = 150 * 1024;

template <typename CT>
static int choose_rb(int CB, int K) {
  if (use_small_k<CT>(K)) {
    // whole runs of rows per thread: RB = RPT x rows per run, at least one
    // row per thread (RB >= kThreads: the runs' adjoint sums reuse the rows'
    // space), at most kSmallRunRows rows per run and ~kSmallTileBytes
    const int rpt = kThreads / CB;
    const size_t row_bytes = sizeof(CT) * (small_row_stride<CT>(K) + 1) + sizeof(int);
    int rr = (int)std::min<size_t>(kSmallRunRows, kSmallTileBytes / (row_bytes * rpt));
    rr = std::max(rr, (kThreads + rpt - 1) / rpt);
    return rr * rpt;
  }
  int rb = 256;
  while (rb > 32 && partial_smem_bytes<CT>(CB, K, rb) > kSmemBudget) rb -= 32;
  return rb;
}

template <typename XT, typename CT, int CB>
static void launch_partial(const ModelDesc& m, const double* Q, int ldq, int C,
                           const int* active, GradWorkspace& ws, cudaStream_t st) {
  const int RB = choose_rb<CT>(CB, m.K);
  const size_t smem = partial_smem_bytes<CT>(CB, m.K, RB);
  if (set_smem_attr<XT, CT, CB>(smem)) return;  // reported by the caller's launch check
  dim3 grid(ws.S, (C + CB - 1) / CB);
  loglik_partial_kernel<XT, CT, CB><<<grid, kThreads, smem, st>>>(
      m, Q, ldq, C, active, ws.split_rows, RB, ws.partial, ws.NP, ws.gz);
}

template <typename XT, typename CT>
static void dispatch_cb(const ModelDesc& m, const double* Q, int ldq, int C,
                        const int* active, GradWorkspace& ws, cudaStream_t st) {
  switch (block_chains(m.K, C)) {
    case 16: launch_partial<XT, CT, 16>(m, Q, ldq, C, active, ws, st); break;
    case 8: launch_partial<XT, CT, 8>(m, Q, ldq, C, active, ws, st); break;
    default: launch_partial<XT, CT, 4>(m, Q, ldq, C, active, ws, st); break;
  }
}

template <typename CT>
static void dispatch_x(const ModelDesc& m, const double* Q, int ldq, int C,
                       const int* active, GradWorkspace& ws, cudaStream_t st) {
  if (m.x_dtype == GBNUTS_F64)
    dispatch_cb<double, CT>(m, Q, ldq, C, active, ws, st);
  else if (m.x_dtype == GBNUTS_F32)
    dispatch_cb<float, CT>(m, Q, ldq, C, active, ws, st);
  else
    dispatch_cb<uint16_t, CT>(m, Q, ldq, C, active, ws, st);
}

int partial_tile_rows(int K, int C, int precision) {
  const int CB = block_chains(K, C);
  return precision == GBNUTS_PREC_FP64 ? choose_rb<double>(CB, K) : choose_rb<float>(CB, K);
}

size_t partial_smem(int K, int C, int rb, int precision) {
  const int CB = block_chains(K, C);
  return precision == GBNUTS_PREC_FP64 ? partial_smem_bytes<double>(CB, K, rb)
                                       : partial_smem_bytes<float>(CB, K, rb);
}

template <typename XT, typename CT, int CB>
static int launch_pool_t(const PoolGradFit* d_fits, const PoolWorkItem* d_items, int n_items,
                         size_t smem, cudaStream_t st) {
  int rc = ensure_smem(loglik_partial_pool_kernel<XT, CT, CB>, smem);
  if (rc) return rc;
  loglik_partial_pool_kernel<XT, CT, CB><<<n_items, kThreads, smem, st>>>(d_fits, d_items);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

template <typename XT, typename CT>
static int launch_pool_cb(const PoolGradFit* d_fits, const PoolWorkItem* d_items, int n_items,
                          int cb, size_t smem, cudaStream_t st) {
  if (cb == 4) return launch_pool_t<XT, CT, 4>(d_fits, d_items, n_items, smem, st);
  if (cb == 8) return launch_pool_t<XT, CT, 8>(d_fits, d_items, n_items, smem, st);
  return launch_pool_t<XT, CT, 16>(d_fits, d_items, n_items, smem, st);
}

int launch_partials_pool(const PoolGradFit* d_fits, const PoolWorkItem* d_items, int n_items,
                         int cb, int x_dtype, int precision, size_t smem, cudaStream_t st) {
  if (n_items <= 0) return GBNUTS_OK;
  const bool f64 = precision == GBNUTS_PREC_FP64;
  if (x_dtype == GBNUTS_F64)
    return f64 ? launch_pool_cb<double, double>(d_fits, d_items, n_items, cb, smem, st)
               : launch_pool_cb<double, float>(d_fits, d_items, n_items, cb, smem, st);
  if (x_dtype == GBNUTS_F32)
    return f64 ? launch_pool_cb<float, double>(d_fits, d_items, n_items, cb, smem, st)
               : launch_pool_cb<float, float>(d_fits, d_items, n_items, cb, smem, st);
  return f64 ? launch_pool_cb<uint16_t, double>(d_fits, d_items, n_items, cb, smem, st)
             : launch_pool_cb<uint16_t, float>(d_fits, d_items, n_items, cb, smem, st);
}

// Minimum rows of a split: the built-in 256 (32 for the FP64 form, whose
// rows cost GB300's FP64 pipe ~20x an FP32 row: a small fit's gradient then
// spreads over more SMs), or the value set through gbnuts_set_launch_shape
// (for tuning).
static std::atomic<long long> g_split_rows_min{0};
void set_split_rows_min(long long rows) { g_split_rows_min.store(rows > 0 ? rows : 0); }
static long long split_rows_min(int precision) {
  const long long r = g_split_rows_min.load();
  return r > 0 ? r : (precision == GBNUTS_PREC_FP64 ? 32LL : 256LL);
}

int choose_splits(const ModelDesc& m, int C, int precision) {
  if (is_tensor_precision(precision)) {
    if (!tc_supported(m))  // wide-design form
      return wide_splits(m, C) * (m.x_dtype == GBNUTS_BF16 ? 1 : 2);
    return tct_splits(m, C);
  }
  const int CB = block_chains(m.K, C);
  const int chain_blocks = (C + CB - 1) / CB;
  // Splits: enough CTAs for ~2 waves over the SMs, a minimum of rows each.
  const int sms = device_sm_count();
  long long max_s = std::max(1LL, m.N / split_rows_min(precision));
  int S = (int)std::min<long long>(max_s, std::max(1, (2 * sms + chain_blocks - 1) / chain_blocks));
  if (m.off_z >= 0) S = std::min(S, m.J);
  S = std::max(S, 1);
  if (precision == GBNUTS_PREC_FP64 && m.off_z < 0) {
    // The FP64 form's CTAs are long (the FP64 pipe) and, with a large tile,
    // one fits per SM: a last wave that is mostly empty costs a whole CTA
    // time.  Among S/2 .. 2S splits (the same minimum of rows each), take the
    // one whose CTAs best fill whole waves, nearest to S on ties.
    const size_t smem = partial_smem(m.K, C, partial_tile_rows(m.K, C, precision), precision);
    const int per_sm = std::max(1, std::min(8, (int)((227u * 1024u) / std::max<size_t>(smem, 1))));
    const long long slots = (long long)sms * per_sm;
    auto fill = [&](int s) {
      const long long ctas = (long long)s * chain_blocks;
      return (double)ctas / (double)(((ctas + slots - 1) / slots) * slots);
    };
    int best = S;
    for (int s = std::max(1, S / 2); s <= 2 * S && s <= max_s; ++s)
      if (fill(s) > fill(best) + 1e-9 || (fill(s) > fill(best) - 1e-9 && abs(s - S) < abs(best - S)))
        best = s;
    S = best;
  }
  return S;
}

int prepare_workspace(const ModelDesc& m, const int* h_group_off, int C, int precision,
                      GradWorkspace& ws) {
  const int CB = chains_per_block(m.K);
  if (CB == 0) {
    set_last_error("K beyond the supported maximum (2048)");
    return GBNUTS_USAGE;
  }
  if (is_tensor_precision(precision) && !tensor_form_supported(m)) {
    set_last_error("the bf16 tensor-core forms need a logistic or Poisson GLM");
    return GBNUTS_USAGE;
  }
  const int S = choose_splits(m, C, precision);
  const int NP = n_partials(m);
  // partial rows: [S][C] in the static layout; a planned narrow tensor-core
  // launch writes at most 128 rows per CTA ([splits][slots])
  const bool dyn = tct_dynamic(m, precision, C);
  const size_t prow = std::max((size_t)S * C, dyn ? (size_t)128 * tct_plan_grid(C) : (size_t)0);
  size_t need = prow * NP * sizeof(double) + (dyn ? (size_t)(2 + C) * sizeof(int) : 0) +
                (m.off_z >= 0 ? (size_t)C * m.J * sizeof(double) : 0) +
                (size_t)(S + 1) * sizeof(long long) + 16;
  if (ws.C == C && ws.S == S && ws.NP == NP && ws.partial && ws.precision == precision)
    return GBNUTS_OK;
  free_workspace(ws);
  ws.C = C;
  ws.S = S;
  ws.NP = NP;
  ws.precision = precision;
  ws.h_split_rows.assign(S + 1, 0);
  for (int s = 0; s <= S; ++s) {
    if (m.off_z >= 0) {
      long long j = (long long)m.J * s / S;
      ws.h_split_rows[s] = h_group_off[j];
    } else {
      ws.h_split_rows[s] = m.N * s / S;
    }
  }
  char* base = nullptr;
  GBN_CUDA_TRY(cudaMalloc(&base, need));
  ws.bytes = need;
  ws.partial = reinterpret_cast<double*>(base);
  size_t off = prow * NP * sizeof(double);
  if (dyn) {
    ws.dyn = reinterpret_cast<int*>(base + off);
    off += (size_t)(2 + C) * sizeof(int);
    off = (off + 7) & ~(size_t)7;
  }
  if (m.off_z >= 0) {
    ws.gz = reinterpret_cast<double*>(base + off);
    off += (size_t)C * m.J * sizeof(double);
  }
  ws.split_rows = reinterpret_cast<long long*>(base + off);
  off += (size_t)(S + 1) * sizeof(long long);
  ws.err = reinterpret_cast<int*>(base + off);
  GBN_CUDA_TRY(cudaMemcpy(ws.split_rows, ws.h_split_rows.data(),
                          (S + 1) * sizeof(long long), cudaMemcpyHostToDevice));
  GBN_CUDA_TRY(cudaMemset(ws.err, 0, sizeof(int)));
  return GBNUTS_OK;
}

void free_workspace(GradWorkspace& ws) {
  if (ws.partial) cudaFree(ws.partial);
  ws = GradWorkspace();
}

int launch_partials(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
                    const int* active, GradWorkspace& ws, cudaStream_t stream, cudaEvent_t ev0,
                    cudaEvent_t ev1) {
  if (m.off_z >= 0)
    GBN_CUDA_TRY(cudaMemsetAsync(ws.gz, 0, (size_t)C * m.J * sizeof(double), stream));
  if (ev0) cudaEventRecord(ev0, stream);
  if (precision == GBNUTS_PREC_FP64) {
    dispatch_x<double>(m, Q, ldq, C, active, ws, stream);
  } else if (precision == GBNUTS_PREC_FP32) {
    dispatch_x<float>(m, Q, ldq, C, active, ws, stream);
  } else if (is_tensor_precision(precision) &&
             (precision == GBNUTS_PREC_F16X3 ? m.tc_xt16 : m.tc_xt) != nullptr) {
    int rc = launch_tct(m, precision, Q, ldq, C, active, ws, stream);
    if (rc) return rc;
  } else if (is_tensor_precision(precision) && m.wide_xt != nullptr) {
    int rc = launch_wide(m, precision, Q, ldq, C, active, ws, stream);
    if (rc) return rc;
  } else {
    set_last_error("precision not available for this model");
    return GBNUTS_USAGE;
  }
  GBN_CUDA_TRY(cudaGetLastError());
  if (ev1) cudaEventRecord(ev1, stream);
  return GBNUTS_OK;
}

int launch_log_prob_grad(const ModelDesc& m, int precision, const double* Q, int ldq,
                         int C, const int* active, double* lp, double* grad, int ldg,
                         int propto, int jacobian, GradWorkspace& ws,
                         cudaStream_t stream, cudaEvent_t ev0, cudaEvent_t ev1) {
  int rc = launch_partials(m, precision, Q, ldq, C, active, ws, stream, ev0, ev1);
  if (rc) return rc;
  // a planned narrow tensor-core launch (active flags given) left its plan
  const int* dyn = (active && ws.dyn && tct_dynamic(m, precision, C)) ? ws.dyn : nullptr;
  loglik_finalize_kernel<<<(C + 3) / 4, 128, 0, stream>>>(m, Q, ldq, C, active, ws.partial,
                                                          ws.NP, ws.S, ws.gz, lp, grad, ldg,
                                                          propto, jacobian, dyn);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

}  // namespace gbn
