// Internal interfaces shared by the gbnuts translation units (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#define GBN_CUDA_TRY(expr)                                                       \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess) {                                                     \
      gbn::set_last_error(std::string(#expr) + ": " + cudaGetErrorString(_e));  \
      return GBNUTS_SOFTWARE;                                                    \
    }                                                                            \
  } while (0)

namespace gbn {

void set_last_error(const std::string& s);
const std::string& last_error();

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device.  Kept per (device, kernel) and guarded by a mutex, so every
// device a process uses gets the opt-in and host threads may launch at once.
int ensure_smem_attr(const void* kernel, size_t bytes);
template <typename F>
inline int ensure_smem(F* kernel, size_t bytes) {
  return ensure_smem_attr(reinterpret_cast<const void*>(kernel), bytes);
}
// Multiprocessor count of the current device (queried once per device).
int device_sm_count();

enum Link { LINK_LOGIT = 0, LINK_POISSON_LOG = 1, LINK_NORMAL = 2 };

// A log density on the device.  theta layout per family:
//   LOGISTIC / POISSON : [alpha], beta[K]
//   HIER_NORMAL        : mu, log tau, log sigma, z[J], beta[K]
//   HIER_LOGISTIC      : alpha, log tau, z[J], beta[K]
// Every family is  eta_n = base + tau z_{g(n)} + x_n . beta  with a link.
struct ModelDesc {
  int kind;
  int link;
  long long N;
  int K, J, D;
  int has_base;   // theta[0] enters eta with coefficient 1
  int idx_tau;    // index of log tau in theta, or -1
  int idx_sigma;  // index of log sigma in theta, or -1
  int off_z;      // first z index, or -1
  int off_beta;   // first beta index
  int x_dtype;    // GBNUTS_F64 / F32 / BF16
  const void* X;  // N x K row-major
  const double* y;
  const int* group;  // N (hierarchical) or nullptr
  double s_base, s_tau, s_sigma, s_beta;  // prior scales
  double r_base2, r_tau2, r_sigma2, r_beta2;  // 1 / scale^2 (set with the scales)
  double sum_lgamma_y;                    // Poisson constant, for propto = false
  // tensor-core forms: X pre-tiled as bf16 hi/lo (128-row tiles), as fp16
  // hi/lo of x 2^tc_x_exp for the f16x3 form, y per tile row
  const void* tc_xt;
  const void* tc_xt16;
  int tc_x_exp;
  const float* tc_yt;
  int tc_tiles;
  // wide-design tensor-core form: X as [tile][slab] 128 x 128 bf16 blocks
  const void* wide_xt;
  int wide_tiles;
};

// Number of per-(split, chain) partial sums: lp, sum r, sum r z_g, sum e^2, beta[K].
inline int n_partials(const ModelDesc& m) { return 4 + m.K; }

// Workspace for one batched gradient evaluation of C chains.
struct GradWorkspace {
  int C = 0, S = 0, NP = 0;
  double* partial = nullptr;   // [S][C][NP]
  double* gz = nullptr;        // [C][J] raw group sums (hierarchical)
  long long* split_rows = nullptr;  // [S+1] device
  int* err = nullptr;               // device error flag of bounded waits
  int precision = -1;
  // theta of the current request as tensor-core words, written by the step
  // kernel during a sampler run (null otherwise)
  const uint32_t* tc_words = nullptr;
  // the narrow tensor-core kernel's plan in a sampler run (see launch_tct):
  // [0] splits, [1] slot stride, [2 + c] chain c's slot; null otherwise
  int* dyn = nullptr;
  std::vector<long long> h_split_rows;
  size_t bytes = 0;
};

// Row splits of a gradient launch for C chains (depends on the model and C
// only, so a fit's sums are the same wherever it runs).
int choose_splits(const ModelDesc& m, int C, int precision);

// Chooses the split count and sets split row boundaries (group aligned for
// hierarchical models).  Allocates (or reuses) the workspace.
int prepare_workspace(const ModelDesc& m, const int* h_group_off, int C, int precision,
                      GradWorkspace& ws);
void free_workspace(GradWorkspace& ws);

// The split partial sums only (no finalize), for callers that finalize
// themselves (the sampler's step kernel).
int launch_partials(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
                    const int* active, GradWorkspace& ws, cudaStream_t stream, cudaEvent_t ev0,
                    cudaEvent_t ev1);

// lp[C] and grad[C][ldg] of C chains at Q[C][ldq] (device pointers), with
// Stan's propto/jacobian semantics; active (may be null) masks chains.
int launch_log_prob_grad(const ModelDesc& m, int precision, const double* Q, int ldq,
                         int C, const int* active, double* lp, double* grad, int ldg,
                         int propto, int jacobian, GradWorkspace& ws,
                         cudaStream_t stream, cudaEvent_t ev0, cudaEvent_t ev1);

// A fit's gradient stage inside a pool launch.
struct PoolGradFit {
  ModelDesc m;
  const double* Q;
  int ldq, C;
  const int* active;
  const long long* split_rows;
  double* P;
  int NP;
  double* Gz;
};
// One CTA of a pool launch.
struct PoolWorkItem {
  int fit, split, chain_block, rb;
};
// Tile rows the partial kernel uses for a given K (same choice as a
// single-fit launch, so a fit's sums do not depend on its pool neighbours).
int partial_tile_rows(int K, int C, int precision);
size_t partial_smem(int K, int C, int rb, int precision);
// Launches the pool partial kernel for work items whose fits share x_dtype
// and block_chains (cb: 4, 8 or 16).
int launch_partials_pool(const PoolGradFit* d_fits, const PoolWorkItem* d_items, int n_items,
                         int cb, int x_dtype, int precision, size_t smem, cudaStream_t st);

// Maximum chains per block of the partial kernel for a given K (0 if K is
// beyond what the kernel supports).
int chains_per_block(int K);
// Device convergence report of a finished fit's draws (lp__ then the
// parameters; rows [row_begin, row_begin + n_rows)): ESS pairs into host
// h_ess[2 x (1 + D)] and/or six-value summaries into h_summary[6 x (1 + D)]
// (either may be null); NaN when the fit is too large for the on-device form.
int fit_ess(const double* d_draws, int C, int max_rows, int n_cols, int row_begin, int n_rows,
            double* h_ess, double* h_summary, cudaStream_t st);

// Chains per block a fit of C chains uses (the smaller of chains_per_block(K)
// and C rounded up to 4, 8 or 16): fewer idle threads for small fits.
int block_chains(int K, int C);

// Tensor-core GLM path, chains on M (Theta and R as tensor-memory operands,
// 128 chains per CTA).  tc_prepare builds the X tiles (f16: the fp16 tiles
// and their scale exponent x_exp) and, when *yt is null, y per tile row.
int tc_prepare(const ModelDesc& m, bool f16, void** xt, float** yt, int* n_tiles, int* x_exp,
               cudaStream_t st);
int tct_splits(const ModelDesc& m, int C);
// Sampler runs of up to kTctPlanMaxChains chains in the narrow tensor-core
// form compact their active chains: the kernel packs the chains that request
// a gradient into as few 128-chain groups as they fill and spreads its CTAs
// over those groups' row splits, so a fit whose chains have partly finished
// takes a shorter launch.  The plan (split count, slot stride, slot of each
// chain) is written to ws.dyn for the step kernel's finalize.
constexpr int kTctPlanMaxChains = 16384;
inline bool tct_dynamic(const ModelDesc& m, int precision, int C);
// CTAs of a planned launch (at least one per 128-chain group).
int tct_plan_grid(int C);
int launch_tct(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
               const int* active, GradWorkspace& ws, cudaStream_t st);
// Minimum rows per split of the CUDA-core gradient (0: the built-in rule).
void set_split_rows_min(long long rows);
// Warps per chain of the step kernel (0: the built-in rule).
void set_team_warps(int w);
// Whether the model can use the tensor-memory kernel (K + intercept <= 128).
inline bool tc_supported(const ModelDesc& m) {
  return (m.link == LINK_LOGIT || m.link == LINK_POISSON_LOG) && m.off_z < 0 &&
         m.K + m.has_base <= 128;
}
// Whether the model has a bf16 tensor-core form at all (GLM families).
inline bool tensor_form_supported(const ModelDesc& m) {
  return (m.link == LINK_LOGIT || m.link == LINK_POISSON_LOG) && m.off_z < 0;
}
inline bool is_tensor_precision(int p) { return p == 2 || p == 3 || p == 4; }
inline bool tct_dynamic(const ModelDesc& m, int precision, int C) {
  return is_tensor_precision(precision) && tc_supported(m) && C <= kTctPlanMaxChains;
}
// Wide-design form (glm_wide.cu, K + intercept > 128): one CTA per (row
// split, 32 chains) with every feature, X in F 128-feature slabs per tile.
// wide_slabs: F (4), 0 when the design is outside the form's range.
// wide_splits: row splits S (the partials then hold S split rows, or 2 S
// when X is not stored in bf16: hi and lo columns of the gradient).
int wide_slabs(const ModelDesc& m);
int wide_splits(const ModelDesc& m, int C);
int wide_prepare(const ModelDesc& m, void** xt, float** yt, int* n_tiles, cudaStream_t st);
int launch_wide(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
                const int* active, GradWorkspace& ws, cudaStream_t st);

}  // namespace gbn
