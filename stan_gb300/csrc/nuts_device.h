// Per-chain sampler state of the device NUTS state machine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbnuts_internal.h"

namespace gbn {

constexpr int MAX_TREE_DEPTH = 16;

// Vector slots of a chain (each `ld` doubles): the two trajectory ends (the
// end being extended is integrated in place), the current sample, the momenta
// at the inner and outer edge of the forward and backward halves, the summed
// momentum, the inverse metric, the Welford accumulators, four scratch
// vectors of the dense metric (A p products), then 6 slots per stack level
// (proposal q, p, g; momentum at the subtree's first and last leaf; summed
// momentum).
enum Slot {
  SL_FWD_Q = 0, SL_FWD_P, SL_FWD_G,
  SL_BCK_Q, SL_BCK_P, SL_BCK_G,
  SL_SMP_Q, SL_SMP_P, SL_SMP_G,
  SL_PFF, SL_PFB, SL_PBF, SL_PBB,
  SL_RHO, SL_INVM, SL_WM, SL_WM2,
  SL_MS0, SL_MS1, SL_MS2, SL_MS3,
  SL_ZNEXT,  // the normals of the next momentum draw, when ChainState::z_ready
  SL_STACK
};

enum Phase {
  PH_INIT_DRAW = 0, PH_INIT_EVAL, PH_SS_BEGIN, PH_SS_TRIAL, PH_SS_EVAL, PH_SS_DONE,
  PH_AFTER_ITER, PH_TRANS_BEGIN, PH_DOUBLING, PH_LEAF_BEGIN, PH_LEAF_EVAL, PH_TRANS_END,
  PH_DONE
};

enum { SS_CTX_START = 0, SS_CTX_WINDOW = 1 };

struct SamplerCfg {
  int C, D, ld, n_slots, max_depth;
  int adapt, num_warmup, num_samples, num_thin, save_warmup;
  int max_rows, n_cols;
  double stepsize, jitter, delta, gamma, kappa, t0, init_radius;
  unsigned wa_num_warmup, wa_init_buffer, wa_term_buffer, wa_base_window;
  unsigned wa_size0, wa_next0;  // window size and end after set_window_params
  unsigned seed, init_chain_id;
  int idx_tau, idx_sigma;
  int dense;  // 1: dense_e metric (FitPtrs::dense), 0: diag_e (slot SL_INVM)
  // Test hook: when set, chain c's uniform #n is script_u[c * script_len + n]
  // and its normal #n script_z[c * script_len + n] (NaN past the end) instead
  // of the counter-based stream (device pointers; null in every other run).
  const double* script_u;
  const double* script_z;
  int script_len;
};

struct ChainState {
  int phase, status, done, iter, init_try;
  int depth, n_lf, divergent, dir, sub_d, leaf;
  int ss_ctx, ss_dir, ss_first, ss_fail;
  int rows, warm_rows, adapt_flag;
  unsigned long long nu, nn;  // uniforms and normals consumed
  long long n_grad, warm_end_ngrad;  // gradients so far; at the end of warmup
  double nom_eps, eps, H0, lsw, sum_metro, accept, energy;
  double V_fwd, V_bck, V_smp, ss_H0;
  double sa_counter, sa_s_bar, sa_x_bar, sa_mu;
  unsigned wa_num_warmup, wa_init_buffer, wa_term_buffer, wa_base_window;
  unsigned wa_counter, wa_next, wa_size;
  double w_n;
  // Work drawn ahead in a short step, off the long path that ends one
  // transition and begins the next: z_ready = the next D normals of the
  // stream (from #nn) are in slot SL_ZNEXT; sa_pre_ready = sqrt and
  // pow(-kappa) of sa_counter + 1 for the next learn_stepsize.
  int z_ready, sa_pre_ready;
  double sa_pre_sqrt, sa_pre_xeta;
};

// Per-level data of the pending left siblings (log sum weight, V of the
// proposal, physical slot of the level), kept apart from ChainState so the
// scalars can live in registers while these are indexed by tree level.
struct ChainStack {
  double lsw[MAX_TREE_DEPTH];
  double V[MAX_TREE_DEPTH];
  int slot[MAX_TREE_DEPTH];
};


// Where the step kernel finds the gradient stage's split partial sums.
struct PartialsView {
  const double* P;
  int NP, S;
  const double* Gz;
  // a planned narrow tensor-core launch's plan (GradWorkspace::dyn), or null
  const int* dyn;
};

// Device pointers of one fit's sampler state and gradient stage.
struct FitPtrs {
  ChainState* states;
  ChainStack* stacks;
  double* vecs;
  double* req;  // positions whose gradient the chains request, [C][ld]
  PartialsView pv;
  int* active;
  double* draws;
  double* diag;
  double* init_out;
  const double* inits;
  int* done_count;
  const int* abort_flag;
  // the request also as chains-on-M tensor-core words (kThetaWords per chain),
  // or null when the gradient form does not read them; req_tc_f16 selects
  // the fp16 words with the chain's scale exponent (the f16x3 form)
  uint32_t* req_tc;
  int req_tc_f16;
  // dense_e: per chain three D x D matrices, column-major (element (i, j) at
  // j * D + i): the inverse metric A, its Cholesky factor L (lower, A = L L^T)
  // and the Welford second-moment sums M2; null for diag_e
  double* dense;
  // Service runs: what the writers need, also written to mapped host memory
  // as it is produced, for the host drain that formats rows while the run
  // goes on (null otherwise).  h_rows / h_diag: as draws / diag; h_count[c]:
  // chain c's rows written; h_init [C][D]; h_adapt [C][1 + M]: the step size
  // at the end of warmup, then the inverse metric (D values, or D x D
  // column-major for dense_e); h_flag[2c] / h_flag[2c + 1]: init / adaptation
  // record written.  Each flag or count is stored after a system-scope fence.
  double* h_rows;
  double* h_diag;
  int* h_count;
  double* h_init;
  double* h_adapt;
  int* h_flag;
};

void launch_nuts_init(const SamplerCfg& cfg, ChainState* states, ChainStack* stacks,
                      double* vecs, const double* inv_metrics, int* active, cudaStream_t s);

// A fit as the step kernel sees it (device-resident table entry).  Single-fit
// runs and pools both launch the step kernel over a table of these.
struct PoolFitDev {
  SamplerCfg cfg;
  ModelDesc m;
  FitPtrs f;
};

// Warps per chain of the step kernel for a dimension D: 1, 2 or 4 (1 up to
// D = 64, 2 up to 1024; gbnuts_set_launch_shape overrides it, for tuning).
int team_warps(int D);

// One step of `total` chains: chain_map[g] = (table index, chain in fit); all
// of them with `team` warps per chain (team_warps of their fit's D).
void launch_nuts_step_pool(const PoolFitDev* fits, const int2* chain_map, int total, int team,
                           cudaStream_t s);

}  // namespace gbn
