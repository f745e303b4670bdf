// Finalisation of one chain's log density and gradient from the split
// partial sums: split sums in a fixed order (deterministic), priors, the
// Jacobian of tau = exp(u), sigma = exp(u), and the chain rule through them.
// One team of threads per chain (team.cuh), threads over the coordinates;
// returns lp in every thread.
// The split sums go through a shared buffer first (split_column_sums).
// Shared by the batched-gradient finalize kernel and the sampler step kernel.
#pragma once

#include <math.h>

#include "gbnuts_internal.h"
#include "team.cuh"

namespace gbn {

static constexpr double kLogSqrt2Pi = 0.91893853320467274178032973640562;

// Largest partial count whose split sums go through the warp's shared buffer.
static constexpr int kMaxColSums = 4 + 512;
// Splits from which the sums run with lanes over splits instead of columns.
static constexpr int kLanesOverSplits = 32;

// Column sums over the S splits of one chain's partials (row stride pstride)
// into cs[k], k < NP.  Lanes over column pairs, as 16-byte loads, when the
// rows are 16-byte aligned and that takes no more rounds of loads than lanes
// over splits; with many splits otherwise: lanes over splits and a fixed
// butterfly per column; else lanes over columns.  Over columns the splits
// are added in split order, their loads issued ten (eight) at a time.  The
// order of additions depends on S, NP and the team size only.
__device__ __forceinline__ void split_column_sums(const double* __restrict__ Pc, size_t pstride,
                                                  int S, int NP, double* cs, const Team& tm) {
  const int pair_rounds = ((NP / 2 + tm.n - 1) / tm.n) * ((S + 9) / 10);
  const int split_rounds = S >= kLanesOverSplits ? (NP + tm.nw - 1) / tm.nw : 1 << 30;
  if (pair_rounds <= split_rounds && ((NP | (int)(pstride & 1)) & 1) == 0 &&
      (reinterpret_cast<uintptr_t>(Pc) & 15) == 0) {
    const int npair = NP >> 1;
    const size_t ps2 = pstride >> 1;
    for (int jb = 0; jb < npair; jb += tm.n) {
      const int j = jb + tm.t;
      if (j < npair) {
        const double2* __restrict__ src = reinterpret_cast<const double2*>(Pc) + j;
        double a0 = 0, a1 = 0;
        for (int s0 = 0; s0 < S; s0 += 10) {
          double2 t[10];
#pragma unroll
          for (int u = 0; u < 10; ++u)
            t[u] = (s0 + u < S) ? src[(size_t)(s0 + u) * ps2] : make_double2(0.0, 0.0);
#pragma unroll
          for (int u = 0; u < 10; ++u)
            if (s0 + u < S) {
              a0 += t[u].x;
              a1 += t[u].y;
            }
        }
        cs[2 * j] = a0;
        cs[2 * j + 1] = a1;
      }
    }
  } else if (S >= kLanesOverSplits) {
    // each warp of the team takes every nw-th column
    const int lane = tm.t & 31;
#pragma unroll 4
    for (int k = tm.t >> 5; k < NP; k += tm.nw) {
      double a = 0;
      for (int s = lane; s < S; s += 32) a += Pc[s * pstride + k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
      if (lane == 0) cs[k] = a;
    }
  } else {
    for (int kb = 0; kb < NP; kb += tm.n) {
      const int k = kb + tm.t;
      double a = 0;
      for (int s0 = 0; s0 < S; s0 += 8) {
        double t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          t[u] = (k < NP && s0 + u < S) ? Pc[(size_t)(s0 + u) * pstride + k] : 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (s0 + u < S) a += t[u];
      }
      if (k < NP) cs[k] = a;
    }
  }
  tm.sync();
}

// th: the chain's parameters; grad_out[d] = sign * d lp / d theta_d.  cs: the
// team's shared buffer of kMaxColSums doubles.  dyn: the plan of a planned
// narrow tensor-core launch (splits, slot stride, slot of each chain), or
// null for partials [S][C][NP].
__device__ __forceinline__ double finalize_chain(const ModelDesc& m, const double* th, int c,
                                                 int C, const double* __restrict__ P, int NP,
                                                 int S, const double* __restrict__ Gz,
                                                 double* grad_out, double sign, int propto,
                                                 int jacobian, const Team& tm, double* cs,
                                                 const int* dyn = nullptr) {
  size_t pstride = (size_t)C * NP;
  const double* Pc = P + (size_t)c * NP;
  if (dyn) {
    S = dyn[0];
    pstride = (size_t)dyn[1] * NP;
    Pc = P + (size_t)dyn[2 + c] * NP;
  }
  const bool use_cs = NP <= kMaxColSums;
  if (use_cs) split_column_sums(Pc, pstride, S, NP, cs, tm);
  // sum over splits of partial column k (split order when lanes run over columns)
  auto col = [&](int k) -> double {
    if (use_cs) return cs[k];
    double a = 0;
#pragma unroll 4
    for (int s = 0; s < S; ++s) a += Pc[s * pstride + k];
    return a;
  };
  const double tau = m.idx_tau >= 0 ? exp(th[m.idx_tau]) : 0.0;
  const double jac = jacobian ? 1.0 : 0.0;
  double prior = 0.0;
  for (int d = tm.t; d < m.D; d += tm.n) {
    const double t = th[d];
    double g;
    if (d >= m.off_beta) {
      const int k = d - m.off_beta;
      const double sum = col(4 + k);
      g = sum - t * m.r_beta2;
      prior += -0.5 * (t * t) * m.r_beta2;
      if (!propto) prior += -log(m.s_beta) - kLogSqrt2Pi;
    } else if (d == 0 && m.has_base) {
      const double sum = col(1);
      g = sum - t * m.r_base2;
      prior += -0.5 * (t * t) * m.r_base2;
      if (!propto) prior += -log(m.s_base) - kLogSqrt2Pi;
    } else if (d == m.idx_tau) {
      const double sum = col(2);
      g = tau * (sum - tau * m.r_tau2) + jac;
      prior += -0.5 * (tau * tau) * m.r_tau2 + jac * t;
      if (!propto) prior += -log(m.s_tau) - kLogSqrt2Pi;
    } else if (d == m.idx_sigma) {
      const double sigma = exp(t);
      const double sum = col(3);
      const double dsig = -(double)m.N / sigma + sum / (sigma * sigma * sigma) -
                          sigma * m.r_sigma2;
      g = sigma * dsig + jac;
      prior += -0.5 * (sigma * sigma) * m.r_sigma2 + jac * t - (double)m.N * t;
      if (!propto) prior += -log(m.s_sigma) - kLogSqrt2Pi;
    } else {  // z_j
      const int j = d - m.off_z;
      g = tau * Gz[(size_t)c * m.J + j] - t;
      prior += -0.5 * t * t;
      if (!propto) prior += -kLogSqrt2Pi;
    }
    grad_out[d] = sign * g;
  }
  prior = tm.sum(prior);
  double lp = col(0) + prior;
  if (!propto) {
    if (m.link == LINK_NORMAL) lp += -(double)m.N * kLogSqrt2Pi;
    if (m.link == LINK_POISSON_LOG) lp += -m.sum_lgamma_y;
  }
  return lp;
}

}  // namespace gbn
