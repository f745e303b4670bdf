// Convergence summaries on the device, one CTA per quantity (a column of the
// draws array), for fits of up to kMaxValues post-warmup draws (chains x draws
// per chain): split rank-normalised bulk and tail ESS and, in the full
// summary, split rank-normalised bulk and tail R-hat and the Monte Carlo
// standard errors of the mean and the sd.  The serving loop's convergence
// report.
//
// Restated from (paths relative to the stan-dev/stan tree):
//   src/stan/analyze/mcmc/split_rank_normalized_ess.hpp:28-55  (bulk, tail)
//   src/stan/analyze/mcmc/split_rank_normalized_rhat.hpp:28-45 (bulk, tail)
//   src/stan/analyze/mcmc/rhat.hpp:20-45                       W and B
//   src/stan/analyze/mcmc/mcse.hpp:22-61                       mcse_mean, mcse_sd
//   src/stan/analyze/mcmc/split_chains.hpp:47-66               halves of each chain
//   src/stan/analyze/mcmc/check_chains.hpp                     finite and varying
//   src/stan/analyze/mcmc/rank_normalization.hpp:23-56         average ranks -> z
//   src/stan/analyze/mcmc/ess.hpp:28-103                       Geyer initial monotone
//   src/stan/analyze/mcmc/autocovariance.hpp:38-99             biased autocovariance
// The autocovariance is summed directly, lag by lag, only as far as Geyer's
// sequence is read (the reference computes every lag by FFT; the values agree
// to round-off).  Sums are block reductions in a fixed order (deterministic).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"

namespace gbn {

namespace {

constexpr int kThreads = 1024;
constexpr int kMaxValues = 8192;  // split draws of one quantity held in shared memory

__device__ double block_sum(double v, double* red) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < nw; ++i) s += red[i];
  return s;
}

// ess.hpp:28-103 on x (m split chains of n draws, chain-major), returns the
// ESS; mean[] and the scratch are shared memory.
__device__ double ess_of(const double* x, int m, int n, double* mean, double* red, int* varies) {
  const int tid = threadIdx.x;
  // A constant chain has a zero lag-0 autocovariance; the reference's FFT
  // autocovariance divides by it and the NaN runs through to tau = 2
  // (autocovariance.hpp:38-99, ess.hpp:28-103): reproduce that outcome.
  for (int j = tid; j < m; j += blockDim.x) varies[j] = 0;
  __syncthreads();
  for (int k = tid; k < m * n; k += blockDim.x) {
    const int j = k / n;
    if (x[k] != x[j * n]) varies[j] = 1;
  }
  __syncthreads();
  int constant = 0;
  for (int j = 0; j < m; ++j) constant |= !varies[j];
  __syncthreads();
  if (constant) return (double)m * n / fmax(2.0, 1.0 / log10((double)m * n));
  // chain means
  for (int j = 0; j < m; ++j) {
    double s = 0.0;
    for (int i = tid; i < n; i += blockDim.x) s += x[j * n + i];
    s = block_sum(s, red);
    if (tid == 0) mean[j] = s / n;
  }
  __syncthreads();
  // mean over chains of the biased autocovariance at lag t
  auto acov_mean = [&](int t) -> double {
    double s = 0.0;
    for (int k = tid; k < m * (n - t); k += blockDim.x) {
      const int j = k / (n - t), i = k - j * (n - t);
      s += (x[j * n + i] - mean[j]) * (x[j * n + i + t] - mean[j]);
    }
    return block_sum(s, red) / n / m;
  };
  const double acov0 = acov_mean(0);
  const double w = acov0 * n / (n - 1);  // mean of the chain variances
  double var_plus = w * (n - 1) / n;
  if (m > 1) {
    double mm = 0.0;
    for (int j = 0; j < m; ++j) mm += mean[j];
    mm /= m;
    double v = 0.0;
    for (int j = 0; j < m; ++j) v += (mean[j] - mm) * (mean[j] - mm);
    var_plus += v / (m - 1);
  }
  // Geyer's initial monotone sequence over pairs of lags; rho[t] for the
  // lags read so far is kept in registers of every thread (identical).
  double rho_even = 1.0;
  double rho_odd = 1.0 - (w - acov_mean(1)) / var_plus;
  double prev_pair = rho_even + rho_odd;  // rho[t-1] + rho[t]
  double sum_rho = rho_even + rho_odd;    // sum of rho[0 .. t]
  double last_kept_even = rho_even;       // rho[t-1] of the last stored pair
  int t = 1;
  while (t < n - 4 && (rho_even + rho_odd > 0) && !isnan(rho_even + rho_odd)) {
    rho_even = 1.0 - (w - acov_mean(t + 1)) / var_plus;
    rho_odd = 1.0 - (w - acov_mean(t + 2)) / var_plus;
    double a = 0.0, b = 0.0;  // rho[t+1], rho[t+2] as stored
    if (rho_even + rho_odd >= 0) {
      a = rho_even;
      b = rho_odd;
    }
    if (a + b > prev_pair) {
      a = prev_pair / 2;
      b = a;
    }
    prev_pair = a + b;
    last_kept_even = a;
    sum_rho += a + b;
    t += 2;
  }
  // sum over rho[0 .. max_t - 1]: drop rho[max_t], the last stored odd lag
  const double s = sum_rho - (prev_pair - last_kept_even);
  const double tail_term = rho_even > 0 ? rho_even : 0.0;
  const double draws_total = (double)m * n;
  double tau = -1.0 + 2.0 * s + tail_term;
  tau = fmax(tau, 1.0 / log10(draws_total));
  return draws_total / tau;
}

// rhat.hpp:20-45 on x (m chains of n draws, chain-major): sqrt of
// ((n - 1) / n W + B / n) / W.
__device__ double rhat_of(const double* x, int m, int n, double* mean, double* red) {
  const int tid = threadIdx.x;
  for (int j = 0; j < m; ++j) {
    double s = 0.0;
    for (int i = tid; i < n; i += blockDim.x) s += x[j * n + i];
    s = block_sum(s, red);
    if (tid == 0) mean[j] = s / n;
  }
  __syncthreads();
  double across = 0.0;
  for (int j = 0; j < m; ++j) across += mean[j];
  across /= m;
  double b = 0.0;
  for (int j = 0; j < m; ++j) b += (mean[j] - across) * (mean[j] - across);
  b = n * b / (m - 1);
  double w = 0.0;
  for (int k = tid; k < m * n; k += blockDim.x) {
    const double d = x[k] - mean[k / n];
    w += d * d;
  }
  w = block_sum(w, red) / (n - 1.0) / m;
  return sqrt((b / w + n - 1) / n);
}

__device__ bool approx_equal(double v, double c) {
  return fabs(v - c) <= 1e-12 * fmin(fabs(v), fabs(c));
}

// bitonic sort of (value, index) pairs, n a power of two
__device__ void bitonic_sort(double* key, int* idx, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const bool up = (i & k) == 0;
          const bool swap = up ? (key[i] > key[l] || (key[i] == key[l] && idx[i] > idx[l]))
                               : (key[i] < key[l] || (key[i] == key[l] && idx[i] < idx[l]));
          if (swap) {
            const double tk = key[i];
            key[i] = key[l];
            key[l] = tk;
            const int ti = idx[i];
            idx[i] = idx[l];
            idx[l] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
}

// average rank of each sorted position of y[0 .. s) (a tie run [a, b] gets
// (a + b) / 2 + 1) -> normal score at the key's original position in x
// (rank_normalization.hpp:23-56)
__device__ void normal_scores(const double* y, const int* idx, int s, double* x) {
  for (int k = threadIdx.x; k < s; k += blockDim.x) {
    int a = k, b = k;
    while (a > 0 && y[a - 1] == y[k]) --a;
    while (b + 1 < s && y[b + 1] == y[k]) ++b;
    const double r = 0.5 * (a + b) + 1.0;
    x[idx[k]] = normcdfinv((r - 0.375) / (s + 0.25));
  }
  __syncthreads();
}

// keys x[0 .. s) padded with +inf to np2, sorted with their positions
__device__ void sort_keys(const double* x, int s, int np2, double* y, int* idx) {
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  for (int k = threadIdx.x; k < np2; k += blockDim.x) {
    y[k] = k < s ? x[k] : inf;
    idx[k] = k;
  }
  __syncthreads();
  bitonic_sort(y, idx, np2);
}

// linear-interpolation (type 7) quantile of the sorted y[0 .. s)
__device__ double sorted_quantile(const double* y, int s, double p) {
  const double at = (s - 1) * p;
  const int lo = (int)floor(at), hi = (int)ceil(at);
  const double f = at - lo;
  return (1 - f) * y[lo] + f * y[hi];
}

// One quantity: draws column q (of n_cols) of C chains, rows [row0, row0 + n).
// FULL: out gets {bulk ESS, tail ESS, bulk R-hat, tail R-hat, mcse_mean,
// mcse_sd} per quantity, else {bulk ESS, tail ESS}.
template <bool FULL>
__global__ void __launch_bounds__(kThreads) summary_kernel(const double* draws, int C,
                                                           int max_rows, int n_cols, int row0,
                                                           int n, int q0, double* out) {
  constexpr int NOUT = FULL ? 6 : 2;
  extern __shared__ unsigned char smem_raw[];
  const int q = q0 + blockIdx.x;
  const int half = n / 2, tail = (n + 1) / 2;
  const int m = 2 * C, s = m * half;
  int np2 = 1;
  while (np2 < s) np2 <<= 1;
  double* x = reinterpret_cast<double*>(smem_raw);  // [s] split draws, chain-major
  double* y = x + kMaxValues;                        // [np2] sort keys / work
  int* idx = reinterpret_cast<int*>(y + kMaxValues);  // [np2]
  __shared__ double red[32];
  __shared__ double mean[2 * 512];
  __shared__ int varies[2 * 512];
  __shared__ int bad;
  double* o = out + (size_t)NOUT * blockIdx.x;
  const int tid = threadIdx.x;
  const double qnan = nan("");
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int k = tid; k < s; k += blockDim.x) {
    const int j = k / half, i = k - j * half;
    const int c = j >> 1;
    const int r = row0 + ((j & 1) ? tail + i : i);
    const double v = draws[((size_t)c * max_rows + r) * n_cols + q];
    x[k] = v;
    if (!isfinite(v)) bad = 1;
  }
  __syncthreads();
  // is_finite_and_varies: no split chain approximately constant, and the
  // chains' first values not all approximately equal
  for (int j = tid; j < m; j += blockDim.x) {
    bool varies = false;
    for (int i = 1; i < half && !varies; ++i) varies = !approx_equal(x[j * half + i], x[j * half]);
    if (!varies) bad = 1;
  }
  if (tid == 0 && m > 1) {
    bool all_eq = true;
    for (int j = 1; j < m && all_eq; ++j) all_eq = approx_equal(x[j * half], x[0]);
    if (all_eq) bad = 1;
  }
  __syncthreads();
  // ESS needs at least 4 draws per split chain; R-hat only finite, varying draws
  const bool ess_ok = !bad && half >= 4;
  if (!bad && (ess_ok || FULL)) {
    // ranks (average over ties, 1-based) -> normal scores
    sort_keys(x, s, np2, y, idx);
    const double q05 = sorted_quantile(y, s, 0.05);
    const double q95 = sorted_quantile(y, s, 0.95);
    const double q50 = sorted_quantile(y, s, 0.5);
    __syncthreads();
    normal_scores(y, idx, s, x);
    const double bulk = ess_ok ? ess_of(x, m, half, mean, red, varies) : qnan;
    __syncthreads();
    double rhat_bulk = qnan;
    if (FULL) {
      rhat_bulk = rhat_of(x, m, half, mean, red);
      __syncthreads();
    }
    double t = qnan;
    if (ess_ok) {
      // tail: indicators of the 5% and 95% quantiles, from the sorted keys'
      // original positions
      for (int k = tid; k < s; k += blockDim.x) x[idx[k]] = y[k] <= q05 ? 1.0 : 0.0;
      __syncthreads();
      const double e05 = ess_of(x, m, half, mean, red, varies);
      __syncthreads();
      for (int k = tid; k < s; k += blockDim.x) x[idx[k]] = y[k] >= q95 ? 1.0 : 0.0;
      __syncthreads();
      const double e95 = ess_of(x, m, half, mean, red, varies);
      __syncthreads();
      if (isnan(e05))
        t = e95;
      else if (isnan(e95))
        t = e05;
      else
        t = fmin(e05, e95);
    }
    double rhat_tail = qnan;
    if (FULL) {
      // distances from the median, ranked again
      for (int k = tid; k < s; k += blockDim.x) x[idx[k]] = fabs(y[k] - q50);
      __syncthreads();
      sort_keys(x, s, np2, y, idx);
      normal_scores(y, idx, s, x);
      rhat_tail = rhat_of(x, m, half, mean, red);
    }
    if (tid == 0) {
      o[0] = bulk;
      o[1] = t;
      if (FULL) {
        o[2] = rhat_bulk;
        o[3] = rhat_tail;
      }
    }
  } else if (tid == 0) {
    for (int j = 0; j < (FULL ? 4 : 2); ++j) o[j] = qnan;
  }
  if (!FULL) return;

  // mcse.hpp:22-61 on the unsplit chains (C chains of n draws, chain-major)
  __syncthreads();
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int k = tid; k < C * n; k += blockDim.x) {
    const int c = k / n, i = k - c * n;
    const double v = draws[((size_t)c * max_rows + row0 + i) * n_cols + q];
    x[k] = v;
    if (!isfinite(v)) bad = 1;
  }
  __syncthreads();
  for (int j = tid; j < C; j += blockDim.x) {
    bool v = false;
    for (int i = 1; i < n && !v; ++i) v = !approx_equal(x[j * n + i], x[j * n]);
    if (!v) bad = 1;
  }
  if (tid == 0 && C > 1) {
    bool all_eq = true;
    for (int j = 1; j < C && all_eq; ++j) all_eq = approx_equal(x[j * n], x[0]);
    if (all_eq) bad = 1;
  }
  __syncthreads();
  if (bad || n < 4) {
    if (tid == 0) o[4] = o[5] = qnan;
    return;
  }
  const double tot = (double)C * n;
  double acc = 0.0;
  for (int k = tid; k < C * n; k += blockDim.x) acc += x[k];
  const double mu = block_sum(acc, red) / tot;
  double a2 = 0.0, a4 = 0.0;
  for (int k = tid; k < C * n; k += blockDim.x) {
    const double d = (x[k] - mu) * (x[k] - mu);
    a2 += d;
    a4 += d * d;
  }
  const double ss = block_sum(a2, red);
  const double s4 = block_sum(a4, red);
  __syncthreads();
  const double e_mean = ess_of(x, C, n, mean, red, varies);
  __syncthreads();
  // ESS of the split chains of |draw - mean|
  for (int k = tid; k < s; k += blockDim.x) {
    const int j = k / half, i = k - j * half;
    const int c = j >> 1;
    const int r = row0 + ((j & 1) ? tail + i : i);
    x[k] = fabs(draws[((size_t)c * max_rows + r) * n_cols + q] - mu);
  }
  __syncthreads();
  const double e_ctr = ess_of(x, m, half, mean, red, varies);
  if (tid == 0) {
    const double evar = ss / tot, fourth = s4 / tot;
    const double varvar = (fourth - evar * evar) / e_ctr;
    o[4] = sqrt(ss / (tot - 1) / e_mean);
    o[5] = sqrt(varvar / evar / 4.0);
  }
}

}  // namespace

}  // namespace gbn

namespace gbn {
namespace {

template <bool FULL>
int launch_summary(const char* who, const double* d_draws, int num_chains, int max_rows,
                   int n_cols, int row_begin, int n_rows, int col_begin, int n_quantities,
                   double* d_out, cudaStream_t st) {
  if (!d_draws || !d_out || num_chains <= 0 || n_rows < 0 || n_quantities <= 0 ||
      col_begin < 0 || col_begin + n_quantities > n_cols || row_begin < 0 ||
      row_begin + n_rows > max_rows) {
    set_last_error(std::string(who) + ": bad arguments");
    return GBNUTS_USAGE;
  }
  const long long held = FULL ? (long long)num_chains * n_rows
                              : 2LL * num_chains * (n_rows / 2);
  if (2 * num_chains > 1024 || held > kMaxValues) {
    set_last_error(std::string(who) + ": more than 8192 draws per quantity");
    return GBNUTS_USAGE;
  }
  const size_t smem = (size_t)kMaxValues * (8 + 8 + 4);
  int rc = ensure_smem(summary_kernel<FULL>, smem);
  if (rc) return rc;
  summary_kernel<FULL><<<n_quantities, kThreads, smem, st>>>(
      d_draws, num_chains, max_rows, n_cols, row_begin, n_rows, col_begin, d_out);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

// host draws -> device, summary, device -> host
template <bool FULL>
int host_summary(const char* who, const double* draws, int num_chains, int max_rows, int n_cols,
                 int row_begin, int n_rows, int col_begin, int n_quantities, double* out) {
  if (!draws || !out || num_chains <= 0 || max_rows < 0 || n_cols <= 0) {
    set_last_error(std::string(who) + ": bad arguments");
    return GBNUTS_USAGE;
  }
  constexpr int NOUT = FULL ? 6 : 2;
  const size_t nd = (size_t)num_chains * max_rows * n_cols;
  double *d_draws = nullptr, *d_out = nullptr;
  GBN_CUDA_TRY(cudaMalloc(&d_draws, nd * sizeof(double)));
  cudaError_t e = cudaMalloc(&d_out, (size_t)NOUT * n_quantities * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpy(d_draws, draws, nd * sizeof(double), cudaMemcpyHostToDevice);
  int rc = GBNUTS_OK;
  if (e == cudaSuccess) {
    rc = launch_summary<FULL>(who, d_draws, num_chains, max_rows, n_cols, row_begin, n_rows,
                              col_begin, n_quantities, d_out, nullptr);
    if (rc == GBNUTS_OK)
      e = cudaMemcpy(out, d_out, (size_t)NOUT * n_quantities * sizeof(double),
                     cudaMemcpyDeviceToHost);
  }
  cudaFree(d_draws);
  cudaFree(d_out);
  if (e != cudaSuccess) {
    set_last_error(std::string(who) + ": " + cudaGetErrorString(e));
    return GBNUTS_SOFTWARE;
  }
  return rc;
}

}  // namespace

// The sampler's own report on a run's draws (lp__ then the D parameters):
// ESS pairs into h_ess and/or the six-value summaries into h_summary (either
// may be null); NaN where the run is outside the kernel's limits.
int fit_ess(const double* d_draws, int C, int max_rows, int n_cols, int row_begin, int n_rows,
            double* h_ess, double* h_summary, cudaStream_t st) {
  const int nq = 1 + (n_cols - 7);
  if (h_ess)
    for (int i = 0; i < 2 * nq; ++i) h_ess[i] = nan("");
  if (h_summary)
    for (int i = 0; i < 6 * nq; ++i) h_summary[i] = nan("");
  const bool fits_split = n_rows >= 8 && 2 * C <= 1024 && 2 * C * (n_rows / 2) <= kMaxValues;
  const bool fits_full = fits_split && (long long)C * n_rows <= kMaxValues;
  const bool do_full = h_summary && fits_full;
  const bool do_ess = h_ess && fits_split;
  if (!do_full && !do_ess) return GBNUTS_OK;
  const int nout = do_full ? 6 : 2;
  double* d_out = nullptr;
  GBN_CUDA_TRY(cudaMalloc(&d_out, (size_t)nout * nq * sizeof(double)));
  auto run = [&](int col, int count, double* dst) {
    return do_full ? launch_summary<true>("fit summary", d_draws, C, max_rows, n_cols, row_begin,
                                          n_rows, col, count, dst, st)
                   : launch_summary<false>("fit ESS", d_draws, C, max_rows, n_cols, row_begin,
                                           n_rows, col, count, dst, st);
  };
  int rc = run(0, 1, d_out);
  if (rc == GBNUTS_OK && nq > 1) rc = run(7, nq - 1, d_out + nout);
  std::vector<double> h((size_t)nout * nq);
  cudaError_t e = cudaSuccess;
  if (rc == GBNUTS_OK)
    e = cudaMemcpyAsync(h.data(), d_out, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_out);
  if (e != cudaSuccess) {
    set_last_error(std::string("fit ESS: ") + cudaGetErrorString(e));
    return GBNUTS_SOFTWARE;
  }
  if (rc != GBNUTS_OK) return rc;
  for (int i = 0; i < nq; ++i) {
    if (do_full) std::copy(&h[6 * i], &h[6 * i] + 6, h_summary + 6 * i);
    if (h_ess && (do_full || do_ess)) {
      h_ess[2 * i] = h[nout * i];
      h_ess[2 * i + 1] = h[nout * i + 1];
    }
  }
  return GBNUTS_OK;
}

}  // namespace gbn

extern "C" int gbnuts_ess_device(const double* d_draws, int num_chains, int max_rows, int n_cols,
                                 int row_begin, int n_rows, int col_begin, int n_quantities,
                                 double* d_out, void* stream) {
  return gbn::launch_summary<false>("gbnuts_ess_device", d_draws, num_chains, max_rows, n_cols,
                                    row_begin, n_rows, col_begin, n_quantities, d_out,
                                    static_cast<cudaStream_t>(stream));
}

extern "C" int gbnuts_summary_device(const double* d_draws, int num_chains, int max_rows,
                                     int n_cols, int row_begin, int n_rows, int col_begin,
                                     int n_quantities, double* d_out, void* stream) {
  return gbn::launch_summary<true>("gbnuts_summary_device", d_draws, num_chains, max_rows,
                                   n_cols, row_begin, n_rows, col_begin, n_quantities, d_out,
                                   static_cast<cudaStream_t>(stream));
}

extern "C" int gbnuts_ess(const double* draws, int num_chains, int max_rows, int n_cols,
                          int row_begin, int n_rows, int col_begin, int n_quantities,
                          double* out) {
  return gbn::host_summary<false>("gbnuts_ess", draws, num_chains, max_rows, n_cols, row_begin,
                                  n_rows, col_begin, n_quantities, out);
}

extern "C" int gbnuts_summary(const double* draws, int num_chains, int max_rows, int n_cols,
                              int row_begin, int n_rows, int col_begin, int n_quantities,
                              double* out) {
  return gbn::host_summary<true>("gbnuts_summary", draws, num_chains, max_rows, n_cols,
                                 row_begin, n_rows, col_begin, n_quantities, out);
}
