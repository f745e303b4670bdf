/*
 * gbnuts: GB300 (sm_103a) NUTS sampling for a fixed family of log densities,
 * behind a plain C ABI (no C++ or CUDA types in any signature).
 *
 * Two groups of entry points stand in for the reference's interfaces
 * (paths relative to the stan-dev/stan tree):
 *
 *  - the model ABI, stan::model::model_base (src/stan/model/model_base.hpp:36-707)
 *    as the sampler reaches it: log_prob / log_prob_grad
 *    (src/stan/model/log_prob_grad.hpp:27-88, log_prob_propto.hpp:31-95,
 *    gradient.hpp:14-35), write_array, unconstrain_array, num_params_r and the
 *    parameter names;
 *  - the service ABI, stan::services::sample::hmc_nuts_diag_e_adapt
 *    (src/stan/services/sample/hmc_nuts_diag_e_adapt.hpp:331-407; single chain
 *    :57-112) and hmc_nuts_diag_e (hmc_nuts_diag_e.hpp:48-100), with the
 *    reference's argument order and its writer / logger / interrupt protocol
 *    (src/stan/callbacks/writer.hpp:16-61, logger.hpp:24-97, interrupt.hpp:14-28,
 *    structured_writer.hpp:16-150) carried by C function pointers.
 *
 * Return codes follow src/stan/services/error_codes.hpp:10-17.  No C++
 * exception crosses this boundary.  Handles are not re-entrant; distinct
 * handles may be used from distinct host threads.
 */
#ifndef GBNUTS_H
#define GBNUTS_H

#ifdef __cplusplus
extern "C" {
#endif

/* error_codes.hpp:10-17 */
enum {
  GBNUTS_OK = 0,
  GBNUTS_USAGE = 64,
  GBNUTS_DATAERR = 65,
  GBNUTS_NOINPUT = 66,
  GBNUTS_SOFTWARE = 70,
  GBNUTS_CONFIG = 78
};

/* Log density families (the models a user of the reference would write as
 * Stan programs; here they are fixed and hand-differentiated). */
enum {
  GBNUTS_LOGISTIC = 1,      /* y ~ bernoulli_logit(alpha + X beta), alpha, beta ~ normal(0, hp0) */
  GBNUTS_POISSON = 2,       /* y ~ poisson_log([alpha +] X beta), coefficients ~ normal(0, hp0) */
  GBNUTS_HIER_NORMAL = 3,   /* y ~ normal(mu + tau z[g] + X beta, sigma), non-centred */
  GBNUTS_HIER_LOGISTIC = 4  /* y ~ bernoulli_logit(alpha + tau z[g] + X beta), non-centred */
};

/* Storage type of X on the device. */
enum { GBNUTS_F64 = 0, GBNUTS_F32 = 1, GBNUTS_BF16 = 2 };

/* Arithmetic of the batched gradient.
 *  FP64   : the plain form; every operation in double precision.
 *  FP32   : X.B and X^T.R in single precision on CUDA cores, per-row link in
 *           single precision, log density total and everything the sampler
 *           does in double precision.
 *  BF16X3 : X.B and X^T.R as bf16 hi/lo split products on the tcgen05 tensor
 *           cores with FP32 accumulation (three products per contraction),
 *           totals and sampler state in double precision.
 *  BF16   : the same contractions as single bf16 products (no lo parts).
 *  F16X3  : the BF16X3 products on fp16 hi/lo parts (22 significant bits per
 *           operand instead of 16, same tensor-core rate), with exact
 *           power-of-two scales keeping every part inside the fp16 range;
 *           logistic GLM with up to 127 features.
 *  The bf16 forms take the logistic and Poisson GLMs: up to 127 features on
 *  the tensor-memory kernel, wider designs as bf16 GEMMs around a link
 *  kernel. */
enum {
  GBNUTS_PREC_FP64 = 0,
  GBNUTS_PREC_FP32 = 1,
  GBNUTS_PREC_BF16X3 = 2,
  GBNUTS_PREC_BF16 = 3,
  GBNUTS_PREC_F16X3 = 4
};

typedef struct gbnuts_model gbnuts_model;

/* ------------------------------------------------------------ model ABI */

/* Creates a model and copies its data to the current CUDA device.
 *   X     : N x K row-major, element type x_dtype (F64 double, F32 float,
 *           BF16 uint16 bit patterns)
 *   y     : N doubles (0/1 for the logistic families, counts for Poisson)
 *   group : N ints in [0, J), non-decreasing (hierarchical families), else NULL
 *   hp    : prior scales, n_hp of them (NULL for the defaults):
 *           LOGISTIC {2.5}; POISSON {1}; HIER_NORMAL {mu 5, tau 1, sigma 1, beta 1};
 *           HIER_LOGISTIC {alpha 2.5, tau 1, beta 2.5}
 * Replaces constructing a generated model_base with its data
 * (model_base.hpp:36-56).  The caller's buffers may be freed on return. */
int gbnuts_model_create(int kind, const void* X, int x_dtype, const double* y,
                        const int* group, long long N, int K, int J, int intercept,
                        const double* hp, int n_hp, gbnuts_model** out);
void gbnuts_model_destroy(gbnuts_model* m);

/* model_base::num_params_r (prob_grad.hpp:57). */
int gbnuts_num_params_r(const gbnuts_model* m);

/* One parameter name: constrained_param_names / unconstrained_param_names
 * (model_base.hpp:129-176), e.g. "beta.3".  Returns the length or -1. */
int gbnuts_param_name(const gbnuts_model* m, int index, int constrained, char* buf,
                      int cap);

/* log_prob<propto, jacobian>(theta) on the unconstrained scale
 * (model_base.hpp:191-203; log_prob_propto.hpp:73-95).  FP64. */
int gbnuts_log_prob(gbnuts_model* m, const double* theta, int propto, int jacobian,
                    double* lp);

/* log_prob_grad<propto, jacobian> (log_prob_grad.hpp:67-88): lp and
 * d lp / d theta for one point, FP64 on the device. */
int gbnuts_log_prob_grad(gbnuts_model* m, const double* theta, int propto,
                         int jacobian, double* lp, double* grad);

/* Batched gradient for C points (host buffers): theta C x D row-major in,
 * lp[C] and grad C x D out, with propto = jacobian = true (the sampler's
 * call, base_hamiltonian.hpp:61-70 via model_functional.hpp:18-23). */
int gbnuts_log_prob_grad_batch(gbnuts_model* m, int C, const double* theta,
                               double* lp, double* grad, int precision);

/* The same with device buffers on the given CUDA stream (cudaStream_t passed
 * as void*; NULL = default stream).  Asynchronous; uses workspace owned by the
 * model handle. */
int gbnuts_log_prob_grad_batch_device(gbnuts_model* m, int C, const double* d_theta,
                                      double* d_lp, double* d_grad, int precision,
                                      void* stream);

/* The batched gradient above without any device allocation.  No counterpart
 * in the reference: it is for callers that cannot allocate device memory when
 * they need a gradient (a host that reserved the device's memory up front for
 * its own pool, code running under another framework's allocator lock, a loop
 * that cannot afford an allocation's implicit synchronisation).  Instead of
 * the handle's workspace it uses one fixed 16 MiB device array in the library;
 * requests needing more (many chains x many features) are rejected with
 * GBNUTS_USAGE.  fp64 and fp32 precisions only.  The first call on each device
 * looks up that array's address and should come before any stream capture.
 * All calls share the array: calls that overlap on the GPU race. */
int gbnuts_log_prob_grad_batch_device_noalloc(gbnuts_model* m, int C, const double* d_theta,
                                              double* d_lp, double* d_grad, int precision,
                                              void* stream);

/* write_array (model_base.hpp:370): unconstrained -> constrained (tau, sigma = exp). */
int gbnuts_write_array(const gbnuts_model* m, const double* theta_unc, double* out);

/* unconstrain_array (model_base.hpp:386): constrained -> unconstrained. */
int gbnuts_unconstrain_array(const gbnuts_model* m, const double* theta, double* out);

/* ------------------------------------------------------------ service ABI */

/* Writer ids passed to the callbacks. */
enum { GBNUTS_INIT_WRITER = 0, GBNUTS_SAMPLE_WRITER = 1, GBNUTS_DIAGNOSTIC_WRITER = 2 };
/* Logger levels (logger.hpp:33-96). */
enum { GBNUTS_DEBUG = 0, GBNUTS_INFO = 1, GBNUTS_WARN = 2, GBNUTS_ERROR = 3, GBNUTS_FATAL = 4 };

/* The reference's callback objects as C function pointers.  Any member may be
 * NULL (the reference's no-op base classes).  writer(names) / writer(values) /
 * writer(message) / writer() are write_names / write_values / write_message /
 * write_blank; logger.{debug..fatal} is log; interrupt() returning nonzero
 * aborts (the interface throwing from interrupt, generate_transitions.hpp:52);
 * structured_writer's {stepsize, metric_type, inv_metric} record
 * (base_hmc.hpp:70-76) is write_metric.  In the service functions the
 * writers receive each chain's init values, names, rows and adaptation block
 * while the device run goes on, from a host drain thread (once every chain
 * has initialised), and the rest (remaining rows, timing, log messages) after
 * it on the calling thread; interrupt is called on the calling thread between
 * step chunks.  With chains_concurrent zero the writers are called from one
 * thread at a time; when it is nonzero, the writers of different chains may be
 * called from different threads at once (each chain's calls stay in order,
 * as in the reference's per-chain TBB tasks), and log must then be
 * thread-safe. */
typedef struct {
  void* ctx;
  void (*write_names)(void* ctx, int chain, int writer, const char* const* names, int n);
  void (*write_values)(void* ctx, int chain, int writer, const double* values, int n);
  void (*write_message)(void* ctx, int chain, int writer, const char* message);
  void (*write_blank)(void* ctx, int chain, int writer);
  void (*log)(void* ctx, int level, const char* message);
  int (*interrupt)(void* ctx);
  void (*write_metric)(void* ctx, int chain, double stepsize, const char* metric_type,
                       const double* inv_metric, int n);
  int want_diagnostics; /* nonzero: the diagnostic writer receives q, p, g rows */
  int chains_concurrent; /* nonzero: chains' writers may run concurrently */
} gbnuts_callbacks;

/* Stan CSV files as the sample and diagnostic writers and JSON files as the
 * metric writer, for num_chains chains with ids chain_id0 + c:
 * <sample_prefix>_<id>.csv, <diagnostic_prefix>_<id>.csv (when not NULL; sets
 * want_diagnostics) and <metric_prefix>_<id>.json (when not NULL).  Rows are
 * stream_writer rows (stream_writer.hpp:16-103: comma-separated, values at
 * sig_figs significant digits as operator<< prints them, "# " before
 * messages); the metric file is json_writer's record (json_writer.hpp,
 * base_hmc.hpp:70-76).  Fills cb (log and interrupt NULL, chains_concurrent
 * set); gbnuts_csv_close flushes and closes every file and reports a failed
 * write.  NOINPUT when a file cannot be created. */
typedef struct gbnuts_csv gbnuts_csv;
int gbnuts_csv_open(const char* sample_prefix, const char* diagnostic_prefix,
                    const char* metric_prefix, int num_chains, int chain_id0, int sig_figs,
                    gbnuts_callbacks* cb, gbnuts_csv** out);
int gbnuts_csv_close(gbnuts_csv* w);

/* hmc_nuts_diag_e_adapt, multi-chain (hmc_nuts_diag_e_adapt.hpp:331-343
 * argument order).  inits: num_chains x D unconstrained values, or NULL for
 * uniform(-init_radius, init_radius) draws; inv_metrics: num_chains x D, or
 * NULL for ones.  Chain i uses chain id init_chain_id + i for its draw stream.
 * precision: GBNUTS_PREC_*.  All chains run in one device run. */
int gbnuts_hmc_nuts_diag_e_adapt(gbnuts_model* m, int num_chains, const double* inits,
                                 const double* inv_metrics, unsigned random_seed,
                                 unsigned init_chain_id, double init_radius,
                                 int num_warmup, int num_samples, int num_thin,
                                 int save_warmup, int refresh, double stepsize,
                                 double stepsize_jitter, int max_depth, double delta,
                                 double gamma, double kappa, double t0,
                                 unsigned init_buffer, unsigned term_buffer,
                                 unsigned window, int precision,
                                 const gbnuts_callbacks* cb);

/* hmc_nuts_dense_e_adapt (hmc_nuts_dense_e_adapt.hpp:57-118 argument order,
 * multi-chain): the same service with a dense metric adapted from the
 * draws' covariance; inv_metrics num_chains x D x D row-major (symmetric
 * positive definite) or NULL for identities.  The adaptation block writes
 * "Elements of inverse mass matrix:" and one message per row; write_metric
 * receives metric_type "dense_e" and n = D * D (row-major). */
int gbnuts_hmc_nuts_dense_e_adapt(gbnuts_model* m, int num_chains, const double* inits,
                                  const double* inv_metrics, unsigned random_seed,
                                  unsigned init_chain_id, double init_radius,
                                  int num_warmup, int num_samples, int num_thin,
                                  int save_warmup, int refresh, double stepsize,
                                  double stepsize_jitter, int max_depth, double delta,
                                  double gamma, double kappa, double t0,
                                  unsigned init_buffer, unsigned term_buffer,
                                  unsigned window, int precision,
                                  const gbnuts_callbacks* cb);

/* hmc_nuts_dense_e (hmc_nuts_dense_e.hpp): dense metric, adaptation off. */
int gbnuts_hmc_nuts_dense_e(gbnuts_model* m, int num_chains, const double* inits,
                            const double* inv_metrics, unsigned random_seed,
                            unsigned init_chain_id, double init_radius, int num_warmup,
                            int num_samples, int num_thin, int save_warmup, int refresh,
                            double stepsize, double stepsize_jitter, int max_depth,
                            int precision, const gbnuts_callbacks* cb);

/* hmc_nuts_diag_e (hmc_nuts_diag_e.hpp:48-60): the same sampler with
 * adaptation off, given step size and inverse metric (the resume path). */
int gbnuts_hmc_nuts_diag_e(gbnuts_model* m, int num_chains, const double* inits,
                           const double* inv_metrics, unsigned random_seed,
                           unsigned init_chain_id, double init_radius, int num_warmup,
                           int num_samples, int num_thin, int save_warmup, int refresh,
                           double stepsize, double stepsize_jitter, int max_depth,
                           int precision, const gbnuts_callbacks* cb);

/* ------------------------------------------------------------ array API */

/* The device run underneath both services, returning arrays instead of
 * writer calls (for interfaces that own their output format). */
typedef struct {
  int num_chains;
  int adapt;              /* 1: adapt_diag_e_nuts, 0: diag_e_nuts */
  int num_warmup, num_samples, num_thin, save_warmup;
  double stepsize, stepsize_jitter;
  int max_depth;
  double delta, gamma, kappa, t0;
  unsigned init_buffer, term_buffer, window;
  double init_radius;
  unsigned random_seed, init_chain_id;
  int precision;
  int save_diagnostics;   /* also keep unconstrained q, p, g per saved row */
  const double* inits;        /* num_chains x D or NULL */
  const double* inv_metrics;  /* num_chains x D (diag_e) or x D x D (dense_e), or NULL */
  int metric;                 /* GBNUTS_METRIC_DIAG or GBNUTS_METRIC_DENSE */
} gbnuts_run_config;

/* Euclidean metrics: diag_e (diag_e_metric.hpp, var_adaptation.hpp) and
 * dense_e (dense_e_metric.hpp, covar_adaptation.hpp).  Dense inverse metrics
 * are row-major D x D per chain, in and out. */
enum { GBNUTS_METRIC_DIAG = 0, GBNUTS_METRIC_DENSE = 1 };

/* Per-chain results.  Row layout (n_cols = 7 + D): lp__, accept_stat__,
 * stepsize__, treedepth__, n_leapfrog__, divergent__, energy__, then the
 * constrained parameters (base_nuts.hpp:206-220, sample.hpp:42-45,
 * mcmc_writer.hpp:63-135).  draws: num_chains x max_rows x n_cols. */
typedef struct {
  int max_rows, n_cols;
  double* draws;          /* caller-allocated: num_chains * max_rows * n_cols */
  double* diagnostics;    /* NULL or num_chains * max_rows * 3D: q, p, g */
  int* n_rows;            /* per chain: rows written */
  int* n_warmup_rows;     /* per chain: of which warmup rows */
  int* status;            /* per chain: GBNUTS_CHAIN_* */
  double* stepsize;       /* per chain: adapted (or given) step size */
  double* inv_metric;     /* num_chains x D (diag_e) or num_chains x D x D (dense_e) */
  double* init;           /* num_chains x D unconstrained init used */
  long long* n_grad;      /* per chain: gradient evaluations */
  double* seconds;        /* num_chains x 2: warmup, sampling (wall clock) */
  /* run totals */
  double total_ms;        /* device run, CUDA events */
  double grad_ms;         /* time in the gradient kernels, CUDA events */
  long long steps;        /* batched gradient steps launched */
  long long kernel_launches;
  /* NULL, or 2 x (1 + D) doubles: split rank-normalised (bulk, tail) ESS of
   * lp__ then of each parameter over the post-warmup draws, computed on the
   * device before the draws are copied out (NaN when a fit has more than 8192
   * split draws per quantity, or where the reference gives NaN). */
  double* ess;
  /* NULL, or 6 x (1 + D) doubles: per quantity (lp__ then each parameter)
   * bulk ESS, tail ESS, bulk R-hat, tail R-hat, mcse_mean, mcse_sd, as
   * gbnuts_summary_device computes them over the post-warmup draws (NaN when
   * the fit holds more than 8192 post-warmup draws per quantity). */
  double* summary;
} gbnuts_run_output;

/* Chain status codes. */
enum {
  GBNUTS_CHAIN_OK = 0,
  GBNUTS_CHAIN_INIT_FAILED = 1,        /* initialize.hpp:214-226 -> CONFIG */
  GBNUTS_CHAIN_STEPSIZE_INIT_FAILED = 2, /* run_adaptive_sampler.hpp:64-67: no draws, OK */
  GBNUTS_CHAIN_STEPSIZE_FAILED = 3,    /* init_stepsize during adaptation -> SOFTWARE */
  GBNUTS_CHAIN_METRIC_OVERFLOW = 4,    /* var_adaptation.hpp:30-36 -> SOFTWARE */
  GBNUTS_CHAIN_INTERRUPTED = 5,
  GBNUTS_CHAIN_BAD_METRIC = 6          /* validate_diag_inv_metric.hpp:18-27 -> CONFIG */
};

int gbnuts_sample_run(gbnuts_model* m, const gbnuts_run_config* cfg,
                      gbnuts_run_output* out, const gbnuts_callbacks* cb);

/* Writes a finished run (cfg and out of gbnuts_sample_run) through the writer
 * callbacks exactly as the service functions do (mcmc_writer.hpp:63-259): per
 * chain the init writer's values, the sample and diagnostic names, warmup
 * rows, "Adaptation terminated" with the step size and inverse metric (and the
 * metric record), sampling rows and the timing block.  The diagnostic writer
 * receives rows only when cb->want_diagnostics is set and out->diagnostics was
 * filled.  With gbnuts_csv_open's callbacks this writes Stan CSV files after a
 * run of the array API or the pool. */
int gbnuts_write_run(const gbnuts_model* m, const gbnuts_run_config* cfg,
                     const gbnuts_run_output* out, const gbnuts_callbacks* cb);

/* ------------------------------------------------------------ fit pool */

/* Continuous batching of many fits on one GPU.  No reference counterpart:
 * the reference's service runs one fit per call
 * (hmc_nuts_diag_e_adapt.hpp:331-407); a pool runs each submitted fit as
 * gbnuts_sample_run would (same draws, same chain status) while every
 * admitted fit shares the step launches.  Forms: GBNUTS_PREC_FP64 / FP32;
 * every fit in a pool stores X as the pool's x_dtype and has K <= 2048. */
typedef struct gbnuts_pool gbnuts_pool;

/* max_fits: fits admitted at once; max_chains: chains admitted at once;
 * reserve_bytes: device memory left free when admitting (a fit is admitted
 * while free memory minus its need stays above this, or when the pool is
 * empty). */
int gbnuts_pool_create(int precision, int x_dtype, int max_fits, long long max_chains,
                       long long reserve_bytes, gbnuts_pool** out);
void gbnuts_pool_destroy(gbnuts_pool* p);

/* Queues a fit: the model arguments of gbnuts_model_create and a run
 * configuration (copied, with its inits / inv_metrics).  out's buffers must
 * stay valid until the fit is done; they are written when it retires. */
int gbnuts_pool_submit(gbnuts_pool* p, int kind, const void* X, int x_dtype, const double* y,
                       const int* group, long long N, int K, int J, int intercept,
                       const double* hp, int n_hp, const gbnuts_run_config* cfg,
                       gbnuts_run_output* out, long long* fit_id);

/* Admits queued fits (FIFO, while a slot, the chain budget and device
 * memory allow), runs n_steps steps of all admitted fits, then retires the
 * fits whose chains have all finished.  Reports fits running / queued. */
int gbnuts_pool_step(gbnuts_pool* p, int n_steps, int* n_running, int* n_queued);

/* state: 0 queued, 1 running, 2 done (*rc = the fit's return code, as
 * gbnuts_sample_run's), 3 unknown id. */
int gbnuts_pool_status(gbnuts_pool* p, long long fit_id, int* state, int* rc);

/* Steps run so far and chains admitted now. */
int gbnuts_pool_stats(gbnuts_pool* p, long long* steps, long long* chains);

/* ------------------------------------------------------------ diagnostics */

/* Split rank-normalised bulk and tail ESS of n_quantities columns
 * [col_begin, col_begin + n_quantities) of a draws array laid out like
 * gbnuts_run_output.draws (num_chains x max_rows x n_cols), over rows
 * [row_begin, row_begin + n_rows) of every chain
 * (split_rank_normalized_ess.hpp:28-55).  out: 2 per quantity (bulk, tail;
 * NaN where the reference returns NaN).  Computed on the device, one CTA per
 * quantity, for up to 8192 split draws per quantity (2 x num_chains x
 * floor(n_rows / 2)).  gbnuts_ess_device takes device buffers and a stream and
 * is asynchronous; gbnuts_ess takes host buffers. */
int gbnuts_ess_device(const double* d_draws, int num_chains, int max_rows, int n_cols,
                      int row_begin, int n_rows, int col_begin, int n_quantities,
                      double* d_out, void* stream);
int gbnuts_ess(const double* draws, int num_chains, int max_rows, int n_cols, int row_begin,
               int n_rows, int col_begin, int n_quantities, double* out);

/* The same columns' full convergence summary, out: 6 per quantity
 *   bulk ESS, tail ESS      split_rank_normalized_ess.hpp:28-55
 *   bulk R-hat, tail R-hat  split_rank_normalized_rhat.hpp:28-45 (rhat.hpp:20-45)
 *   mcse_mean, mcse_sd      mcse.hpp:22-61 (on the unsplit chains)
 * NaN where the reference returns NaN.  For up to 8192 draws per quantity
 * (num_chains x n_rows) and 512 chains.  Device and host-buffer forms as above. */
int gbnuts_summary_device(const double* d_draws, int num_chains, int max_rows, int n_cols,
                          int row_begin, int n_rows, int col_begin, int n_quantities,
                          double* d_out, void* stream);
int gbnuts_summary(const double* draws, int num_chains, int max_rows, int n_cols, int row_begin,
                   int n_rows, int col_begin, int n_quantities, double* out);

/* Launch-shape overrides, for tuning (no counterpart in the reference).
 * Process-wide; 0 restores the built-in rule.  split_rows_min: minimum rows
 * per row split of the CUDA-core gradient (fp64 / fp32 forms); team_warps:
 * warps per chain of the step kernel (1, 2, 4 or 8).  A fit's splits fix the
 * order of its gradient sums, so a setting changes draws at round-off level
 * (runs stay deterministic for a fixed setting); change it between runs, not
 * while one is going.  USAGE for a team_warps other than 0, 1, 2, 4, 8. */
int gbnuts_set_launch_shape(long long split_rows_min, int team_warps);

/* Device and build information: writes a short text description. */
int gbnuts_device_info(char* buf, int cap);

/* Message of the last failing call on this thread (empty if none). */
int gbnuts_last_error(char* buf, int cap);

#ifdef __cplusplus
}
#endif
#endif /* GBNUTS_H */
