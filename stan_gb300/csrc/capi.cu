// The C ABI of gbnuts: model handles (the model_base stand-in), the batched
// gradient entry points, the device run loop and the two sampling services
// with the reference's writer / logger / interrupt protocol.
//
// Service protocol restated from (paths relative to the stan-dev/stan tree):
//   src/stan/services/sample/hmc_nuts_diag_e_adapt.hpp:331-407 (set-up, error codes)
//   src/stan/services/sample/hmc_nuts_diag_e.hpp:48-100
//   src/stan/services/util/run_adaptive_sampler.hpp:46-103, run_sampler.hpp
//   src/stan/services/util/mcmc_writer.hpp:63-259 (names, rows, adaptation, timing)
//   src/stan/mcmc/windowed_adaptation.hpp:29-78 (set_window_params and its messages)
//   src/stan/services/util/initialize.hpp:68-227 (init messages)
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <sstream>
#include <string>
#include <vector>
#include <thread>
#include <atomic>
#include <map>
#include <mutex>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"
#include "nuts_device.h"
#include "capi_internal.h"
#include "tc_common.cuh"

namespace gbn {
static thread_local std::string g_last_error;
void set_last_error(const std::string& s) { g_last_error = s; }
const std::string& last_error() { return g_last_error; }

static std::mutex g_dev_mu;

int ensure_smem_attr(const void* kernel, size_t bytes) {
  int dev = 0;
  GBN_CUDA_TRY(cudaGetDevice(&dev));
  static std::map<std::pair<int, const void*>, size_t> done;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  size_t& have = done[{dev, kernel}];
  if (bytes > have) {
    GBN_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)bytes));
    have = bytes;
  }
  return GBNUTS_OK;
}

int device_sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  static std::map<int, int> count;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  auto it = count.find(dev);
  if (it != count.end()) return it->second;
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    n = 1;
  count[dev] = n;
  return n;
}
}  // namespace gbn

using namespace gbn;

// Builds the tensor-core tiles of X on first use of a tensor-core form.
static int ensure_precision(gbnuts_model* m, int precision) {
  if (precision < GBNUTS_PREC_FP64 || precision > GBNUTS_PREC_F16X3)
    return fail(GBNUTS_USAGE, "unknown precision");
  if (!is_tensor_precision(precision)) return GBNUTS_OK;
  if (precision == GBNUTS_PREC_F16X3) {
    if (m->desc.link != LINK_LOGIT || !tc_supported(m->desc))
      return fail(GBNUTS_USAGE,
                  "the f16x3 form takes the logistic GLM with up to 127 features");
    if (m->d_tc_xt16) return GBNUTS_OK;
    int tiles = 0, x_exp = 0;
    int rc = tc_prepare(m->desc, true, &m->d_tc_xt16, &m->d_tc_yt, &tiles, &x_exp, m->stream);
    if (rc) return rc;
    GBN_CUDA_TRY(cudaStreamSynchronize(m->stream));
    m->desc.tc_xt16 = m->d_tc_xt16;
    m->desc.tc_x_exp = x_exp;
    m->desc.tc_yt = m->d_tc_yt;
    m->desc.tc_tiles = tiles;
    return GBNUTS_OK;
  }
  if (!tc_supported(m->desc) && tensor_form_supported(m->desc)) {
    // wide design: X as slab tiles for the wide-design kernel
    if (m->d_wide_xt) return GBNUTS_OK;
    int tiles = 0;
    int rc = wide_prepare(m->desc, &m->d_wide_xt, &m->d_tc_yt, &tiles, m->stream);
    if (rc) return rc;
    GBN_CUDA_TRY(cudaStreamSynchronize(m->stream));
    m->desc.wide_xt = m->d_wide_xt;
    m->desc.wide_tiles = tiles;
    m->desc.tc_yt = m->d_tc_yt;
    return GBNUTS_OK;
  }
  if (!tc_supported(m->desc))
    return fail(GBNUTS_USAGE,
                "the bf16 tensor-core forms need a logistic or Poisson GLM");
  if (m->d_tc_xt) return GBNUTS_OK;
  int tiles = 0, x_exp = 0;
  int rc = tc_prepare(m->desc, false, &m->d_tc_xt, &m->d_tc_yt, &tiles, &x_exp, m->stream);
  if (rc) return rc;
  GBN_CUDA_TRY(cudaStreamSynchronize(m->stream));
  m->desc.tc_xt = m->d_tc_xt;
  m->desc.tc_yt = m->d_tc_yt;
  m->desc.tc_tiles = tiles;
  return GBNUTS_OK;
}

static int check_device_error(GradWorkspace& ws) {
  if (!ws.err) return GBNUTS_OK;
  int e = 0;
  GBN_CUDA_TRY(cudaMemcpy(&e, ws.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(ws.err, 0, sizeof(int));
    return fail(GBNUTS_SOFTWARE, "a device wait timed out (code " + std::to_string(e) + ")");
  }
  return GBNUTS_OK;
}

static void host_names(const ModelDesc& m, bool constrained_unused, std::vector<std::string>& out) {
  (void)constrained_unused;
  out.clear();
  if (m.kind == GBNUTS_LOGISTIC || m.kind == GBNUTS_POISSON) {
    if (m.has_base) out.push_back("alpha");
  } else if (m.kind == GBNUTS_HIER_NORMAL) {
    out.push_back("mu");
    out.push_back("tau");
    out.push_back("sigma");
  } else {
    out.push_back("alpha");
    out.push_back("tau");
  }
  for (int j = 0; j < (m.off_z >= 0 ? m.J : 0); ++j) out.push_back("z." + std::to_string(j + 1));
  for (int k = 0; k < m.K; ++k) out.push_back("beta." + std::to_string(k + 1));
}

static int ensure_scratch(gbnuts_model* m, int C) {
  if (m->scratch_C >= C) return GBNUTS_OK;
  if (m->d_theta) cudaFree(m->d_theta);
  m->d_theta = nullptr;
  const size_t D = m->desc.D;
  char* base = nullptr;
  GBN_CUDA_TRY(cudaMalloc(&base, (size_t)C * (2 * D + 1) * sizeof(double)));
  m->d_theta = reinterpret_cast<double*>(base);
  m->d_grad = m->d_theta + (size_t)C * D;
  m->d_lp = m->d_grad + (size_t)C * D;
  m->scratch_C = C;
  return GBNUTS_OK;
}

// Draws of the next gbnuts_sample_run on this thread, when a test sets them
// (gbnuts_sample_run_scripted): num_chains x len uniforms and normals.
static thread_local struct {
  const double* u = nullptr;
  const double* z = nullptr;
  int len = 0;
} g_draw_script;

// Mapped host arrays of the service's host drain for the next
// gbnuts_sample_run on this thread (device-side pointers), or null.
struct DrainPtrs {
  double* rows;
  double* diag;
  int* count;
  double* init;
  double* adapt;
  int* flag;
};
static thread_local const DrainPtrs* g_drain = nullptr;

// Read-only view of a model for the no-allocation entry point (noalloc.cu).
int gbnuts_internal_model_view(const gbnuts_model* m, gbn::ModelDesc* desc,
                               const int** group_off) {
  if (!m) return fail(GBNUTS_USAGE, "model is NULL");
  *desc = m->desc;
  *group_off = m->h_group_off.empty() ? nullptr : m->h_group_off.data();
  return GBNUTS_OK;
}

extern "C" {

int gbnuts_sample_run_scripted(gbnuts_model* m, const gbnuts_run_config* cfg,
                               gbnuts_run_output* out, const double* uniforms,
                               const double* normals, int n_per_chain) {
  if (!uniforms || !normals || n_per_chain <= 0)
    return fail(GBNUTS_USAGE, "scripted draws: uniforms, normals and a positive length");
  g_draw_script.u = uniforms;
  g_draw_script.z = normals;
  g_draw_script.len = n_per_chain;
  const int rc = gbnuts_sample_run(m, cfg, out, nullptr);
  g_draw_script.len = 0;
  g_draw_script.u = g_draw_script.z = nullptr;
  return rc;
}

int gbnuts_set_launch_shape(long long split_rows_min, int team_warps) {
  if (split_rows_min < 0 || !(team_warps == 0 || team_warps == 1 || team_warps == 2 ||
                              team_warps == 4 || team_warps == 8))
    return fail(GBNUTS_USAGE, "split_rows_min >= 0 and team_warps in {0, 1, 2, 4, 8}");
  set_split_rows_min(split_rows_min);
  set_team_warps(team_warps);
  return GBNUTS_OK;
}

int gbnuts_last_error(char* buf, int cap) {
  if (!buf || cap <= 0) return -1;
  strncpy(buf, g_last_error.c_str(), cap - 1);
  buf[cap - 1] = 0;
  return (int)g_last_error.size();
}

int gbnuts_device_info(char* buf, int cap) {
  int dev = 0, rt = 0, drv = 0;
  cudaDeviceProp p;
  std::ostringstream s;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
    s << "no CUDA device";
  } else {
    cudaRuntimeGetVersion(&rt);
    cudaDriverGetVersion(&drv);
    s << p.name << " sm_" << p.major << p.minor << " SMs=" << p.multiProcessorCount
      << " runtime=" << rt << " driver=" << drv;
  }
  std::string str = s.str();
  if (buf && cap > 0) {
    strncpy(buf, str.c_str(), cap - 1);
    buf[cap - 1] = 0;
  }
  return (int)str.size();
}

int gbnuts_model_create(int kind, const void* X, int x_dtype, const double* y,
                        const int* group, long long N, int K, int J, int intercept,
                        const double* hp, int n_hp, gbnuts_model** out) {
  if (!out) return fail(GBNUTS_USAGE, "out is NULL");
  *out = nullptr;
  if (kind < GBNUTS_LOGISTIC || kind > GBNUTS_HIER_LOGISTIC)
    return fail(GBNUTS_USAGE, "unknown model kind");
  if (x_dtype < GBNUTS_F64 || x_dtype > GBNUTS_BF16) return fail(GBNUTS_USAGE, "unknown x_dtype");
  if (N <= 0 || K < 0 || (K > 0 && !X) || !y) return fail(GBNUTS_DATAERR, "bad data shape");
  if (chains_per_block(K) == 0) return fail(GBNUTS_USAGE, "K above 2048 is not supported");
  const bool hier = kind == GBNUTS_HIER_NORMAL || kind == GBNUTS_HIER_LOGISTIC;
  if (hier && (J <= 0 || !group)) return fail(GBNUTS_DATAERR, "hierarchical model needs J > 0 and group");
  // data checks (DATAERR): finite X and y, valid 0/1 or count y, sorted groups
  const size_t NK = (size_t)N * K;
  for (size_t i = 0; i < NK; ++i) {
    double v;
    if (x_dtype == GBNUTS_F64)
      v = static_cast<const double*>(X)[i];
    else if (x_dtype == GBNUTS_F32)
      v = static_cast<const float*>(X)[i];
    else {
      uint32_t b = ((uint32_t) static_cast<const uint16_t*>(X)[i]) << 16;
      float f;
      memcpy(&f, &b, 4);
      v = f;
    }
    if (!isfinite(v)) return fail(GBNUTS_DATAERR, "X has a non-finite value");
  }
  double sum_lgamma = 0.0;
  for (long long n = 0; n < N; ++n) {
    double v = y[n];
    if (!isfinite(v)) return fail(GBNUTS_DATAERR, "y has a non-finite value");
    if ((kind == GBNUTS_LOGISTIC || kind == GBNUTS_HIER_LOGISTIC) && v != 0.0 && v != 1.0)
      return fail(GBNUTS_DATAERR, "logistic y must be 0 or 1");
    if (kind == GBNUTS_POISSON) {
      if (v < 0 || v != floor(v)) return fail(GBNUTS_DATAERR, "Poisson y must be counts");
      sum_lgamma += lgamma(v + 1.0);
    }
  }
  std::vector<int> off;
  if (hier) {
    off.assign(J + 1, 0);
    int prev = -1;
    for (long long n = 0; n < N; ++n) {
      int g = group[n];
      if (g < 0 || g >= J) return fail(GBNUTS_DATAERR, "group index out of range");
      if (g < prev) return fail(GBNUTS_DATAERR, "rows must be sorted by group");
      prev = g;
      off[g + 1]++;
    }
    for (int j = 0; j < J; ++j) off[j + 1] += off[j];
  }
  gbnuts_model* m = new gbnuts_model();
  ModelDesc& d = m->desc;
  memset(&d, 0, sizeof(d));
  d.kind = kind;
  d.N = N;
  d.K = K;
  d.J = hier ? J : 0;
  d.x_dtype = x_dtype;
  d.idx_tau = d.idx_sigma = d.off_z = -1;
  auto hpv = [&](int i, double dflt) { return (hp && i < n_hp) ? hp[i] : dflt; };
  switch (kind) {
    case GBNUTS_LOGISTIC:
    case GBNUTS_POISSON:
      d.link = kind == GBNUTS_LOGISTIC ? LINK_LOGIT : LINK_POISSON_LOG;
      d.has_base = intercept ? 1 : 0;
      d.off_beta = d.has_base;
      d.D = K + d.has_base;
      d.s_base = d.s_beta = hpv(0, kind == GBNUTS_LOGISTIC ? 2.5 : 1.0);
      break;
    case GBNUTS_HIER_NORMAL:
      d.link = LINK_NORMAL;
      d.has_base = 1;
      d.idx_tau = 1;
      d.idx_sigma = 2;
      d.off_z = 3;
      d.off_beta = 3 + J;
      d.D = 3 + J + K;
      d.s_base = hpv(0, 5.0);
      d.s_tau = hpv(1, 1.0);
      d.s_sigma = hpv(2, 1.0);
      d.s_beta = hpv(3, 1.0);
      break;
    default:
      d.link = LINK_LOGIT;
      d.has_base = 1;
      d.idx_tau = 1;
      d.off_z = 2;
      d.off_beta = 2 + J;
      d.D = 2 + J + K;
      d.s_base = hpv(0, 2.5);
      d.s_tau = hpv(1, 1.0);
      d.s_beta = hpv(2, 2.5);
      break;
  }
  d.sum_lgamma_y = sum_lgamma;
  d.r_base2 = 1.0 / (d.s_base * d.s_base);
  d.r_tau2 = 1.0 / (d.s_tau * d.s_tau);
  d.r_sigma2 = 1.0 / (d.s_sigma * d.s_sigma);
  d.r_beta2 = 1.0 / (d.s_beta * d.s_beta);
  const size_t xbytes = NK * (x_dtype == GBNUTS_F64 ? 8 : x_dtype == GBNUTS_F32 ? 4 : 2);
  cudaError_t e = cudaSuccess;
  if (xbytes) e = cudaMalloc(&m->d_X, xbytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_y, N * sizeof(double));
  if (e == cudaSuccess && hier) e = cudaMalloc(&m->d_group, N * sizeof(int));
  if (e == cudaSuccess && xbytes) e = cudaMemcpy(m->d_X, X, xbytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_y, y, N * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && hier)
    e = cudaMemcpy(m->d_group, group, N * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    gbnuts_model_destroy(m);
    return fail(GBNUTS_SOFTWARE, std::string("device allocation: ") + cudaGetErrorString(e));
  }
  d.X = m->d_X;
  d.y = m->d_y;
  d.group = m->d_group;
  m->h_group_off = off;
  *out = m;
  return GBNUTS_OK;
}

void gbnuts_model_destroy(gbnuts_model* m) {
  if (!m) return;
  free_workspace(m->ws);
  if (m->d_tc_xt) cudaFree(m->d_tc_xt);
  if (m->d_tc_xt16) cudaFree(m->d_tc_xt16);
  if (m->d_tc_yt) cudaFree(m->d_tc_yt);
  if (m->d_wide_xt) cudaFree(m->d_wide_xt);
  if (m->d_theta) cudaFree(m->d_theta);
  if (m->d_X) cudaFree(m->d_X);
  if (m->d_y) cudaFree(m->d_y);
  if (m->d_group) cudaFree(m->d_group);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

int gbnuts_num_params_r(const gbnuts_model* m) { return m ? m->desc.D : -1; }

int gbnuts_param_name(const gbnuts_model* m, int index, int constrained, char* buf, int cap) {
  if (!m || index < 0 || index >= m->desc.D) return -1;
  std::vector<std::string> names;
  host_names(m->desc, constrained != 0, names);
  const std::string& s = names[index];
  if (buf && cap > 0) {
    strncpy(buf, s.c_str(), cap - 1);
    buf[cap - 1] = 0;
  }
  return (int)s.size();
}

static int eval_points(gbnuts_model* m, int C, const double* theta, int propto, int jacobian,
                       double* lp, double* grad, int precision) {
  if (!m || C <= 0 || !theta) return fail(GBNUTS_USAGE, "bad arguments");
  const int D = m->desc.D;
  int rc = ensure_precision(m, precision);
  if (rc) return rc;
  rc = ensure_scratch(m, C);
  if (rc) return rc;
  rc = prepare_workspace(m->desc, m->h_group_off.data(), C, precision, m->ws);
  if (rc) return rc;
  GBN_CUDA_TRY(cudaMemcpyAsync(m->d_theta, theta, (size_t)C * D * sizeof(double),
                               cudaMemcpyHostToDevice, m->stream));
  rc = launch_log_prob_grad(m->desc, precision, m->d_theta, D, C, nullptr, m->d_lp, m->d_grad,
                            D, propto, jacobian, m->ws, m->stream, nullptr, nullptr);
  if (rc) return rc;
  GBN_CUDA_TRY(cudaMemcpyAsync(lp, m->d_lp, C * sizeof(double), cudaMemcpyDeviceToHost,
                               m->stream));
  if (grad)
    GBN_CUDA_TRY(cudaMemcpyAsync(grad, m->d_grad, (size_t)C * D * sizeof(double),
                                 cudaMemcpyDeviceToHost, m->stream));
  GBN_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return check_device_error(m->ws);
}

int gbnuts_log_prob_grad_batch_active(gbnuts_model* m, const double* theta, int num_points,
                                      const int* active, int precision, double* lp,
                                      double* grad) {
  if (!m || num_points <= 0 || !theta || !active || !lp || !grad)
    return fail(GBNUTS_USAGE, "bad arguments");
  const int C = num_points, D = m->desc.D;
  int rc = ensure_precision(m, precision);
  if (rc) return rc;
  rc = ensure_scratch(m, C);
  if (rc) return rc;
  rc = prepare_workspace(m->desc, m->h_group_off.data(), C, precision, m->ws);
  if (rc) return rc;
  int* d_active = nullptr;
  GBN_CUDA_TRY(cudaMalloc(&d_active, (size_t)C * sizeof(int)));
  struct Free {
    int* p;
    ~Free() { cudaFree(p); }
  } guard{d_active};
  GBN_CUDA_TRY(cudaMemcpyAsync(d_active, active, (size_t)C * sizeof(int), cudaMemcpyHostToDevice,
                               m->stream));
  GBN_CUDA_TRY(cudaMemcpyAsync(m->d_theta, theta, (size_t)C * D * sizeof(double),
                               cudaMemcpyHostToDevice, m->stream));
  rc = launch_log_prob_grad(m->desc, precision, m->d_theta, D, C, d_active, m->d_lp, m->d_grad,
                            D, 1, 1, m->ws, m->stream, nullptr, nullptr);
  if (rc) return rc;
  GBN_CUDA_TRY(cudaMemcpyAsync(lp, m->d_lp, C * sizeof(double), cudaMemcpyDeviceToHost,
                               m->stream));
  GBN_CUDA_TRY(cudaMemcpyAsync(grad, m->d_grad, (size_t)C * D * sizeof(double),
                               cudaMemcpyDeviceToHost, m->stream));
  GBN_CUDA_TRY(cudaStreamSynchronize(m->stream));
  return check_device_error(m->ws);
}

int gbnuts_log_prob(gbnuts_model* m, const double* theta, int propto, int jacobian,
                    double* lp) {
  if (!lp) return fail(GBNUTS_USAGE, "lp is NULL");
  return eval_points(m, 1, theta, propto, jacobian, lp, nullptr, GBNUTS_PREC_FP64);
}

int gbnuts_log_prob_grad(gbnuts_model* m, const double* theta, int propto, int jacobian,
                         double* lp, double* grad) {
  if (!lp || !grad) return fail(GBNUTS_USAGE, "lp or grad is NULL");
  return eval_points(m, 1, theta, propto, jacobian, lp, grad, GBNUTS_PREC_FP64);
}

int gbnuts_log_prob_grad_batch(gbnuts_model* m, int C, const double* theta, double* lp,
                               double* grad, int precision) {
  if (!lp || !grad) return fail(GBNUTS_USAGE, "lp or grad is NULL");
  return eval_points(m, C, theta, 1, 1, lp, grad, precision);
}

int gbnuts_log_prob_grad_batch_device(gbnuts_model* m, int C, const double* d_theta,
                                      double* d_lp, double* d_grad, int precision,
                                      void* stream) {
  if (!m || C <= 0 || !d_theta || !d_lp || !d_grad) return fail(GBNUTS_USAGE, "bad arguments");
  int rc = ensure_precision(m, precision);
  if (rc) return rc;
  rc = prepare_workspace(m->desc, m->h_group_off.data(), C, precision, m->ws);
  if (rc) return rc;
  return launch_log_prob_grad(m->desc, precision, d_theta, m->desc.D, C, nullptr, d_lp, d_grad,
                              m->desc.D, 1, 1, m->ws, static_cast<cudaStream_t>(stream),
                              nullptr, nullptr);
}

int gbnuts_write_array(const gbnuts_model* m, const double* th, double* out) {
  if (!m || !th || !out) return fail(GBNUTS_USAGE, "bad arguments");
  for (int d = 0; d < m->desc.D; ++d) {
    double v = th[d];
    if (d == m->desc.idx_tau || d == m->desc.idx_sigma) v = exp(v);
    out[d] = v;
  }
  return GBNUTS_OK;
}

int gbnuts_unconstrain_array(const gbnuts_model* m, const double* th, double* out) {
  if (!m || !th || !out) return fail(GBNUTS_USAGE, "bad arguments");
  for (int d = 0; d < m->desc.D; ++d) {
    double v = th[d];
    if (d == m->desc.idx_tau || d == m->desc.idx_sigma) {
      if (!(v > 0)) return fail(GBNUTS_DATAERR, "positive parameter is not positive");
      v = log(v);
    }
    out[d] = v;
  }
  return GBNUTS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ the run
namespace {

struct WindowParams {
  unsigned num_warmup = 0, init_buffer = 0, term_buffer = 0, base_window = 0;
  unsigned size0 = 0, next0 = 0;
  std::vector<std::string> messages;
};

// windowed_adaptation::set_window_params (windowed_adaptation.hpp:29-78), on
// a freshly constructed adapter whose restart() left size 0 and end index
// 0 + 0 - 1 (unsigned).
WindowParams window_params(unsigned nw, unsigned ib, unsigned tb, unsigned bw) {
  WindowParams w;
  w.size0 = 0;
  w.next0 = 0u + 0u - 1u;
  if (nw < 20) {
    w.messages = {"WARNING: No variance estimation is", "         performed for num_warmup < 20",
                  ""};
    return w;
  }
  if (ib + bw + tb > nw) {
    w.num_warmup = nw;
    w.init_buffer = (unsigned)(0.15 * nw);
    w.term_buffer = (unsigned)(0.1 * nw);
    w.base_window = nw - (w.init_buffer + w.term_buffer);
    std::ostringstream a, b, c;
    a << "           init_buffer = " << w.init_buffer;
    b << "           adapt_window = " << w.base_window;
    c << "           term_buffer = " << w.term_buffer;
    w.messages = {"WARNING: There aren't enough warmup iterations to fit the",
                  "         three stages of adaptation as currently configured.",
                  "         Reducing each adaptation stage to 15%/75%/10% of",
                  "         the given number of warmup iterations:",
                  a.str(), b.str(), c.str(), ""};
    return w;
  }
  w.num_warmup = nw;
  w.init_buffer = ib;
  w.term_buffer = tb;
  w.base_window = bw;
  w.size0 = bw;
  w.next0 = ib + bw - 1u;
  return w;
}

struct DeviceRun {
  std::vector<void*> allocs;
  ~DeviceRun() {
    for (void* p : allocs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t n) {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) allocs.push_back(v);
    *p = static_cast<T*>(v);
    return e;
  }
};

// L (row-major, lower) with a = L L^T from the lower triangle of the
// row-major n x n matrix a, column by column with every dot product summed in
// ascending k, as the step kernel factors adapted metrics; false when a pivot
// is not positive.
bool host_cholesky(const double* a, int n, std::vector<double>& l) {
  l.assign((size_t)n * n, 0.0);
  std::vector<double> s(n);
  for (int j = 0; j < n; ++j) {
    for (int i = j; i < n; ++i) {
      double v = a[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) v = v - l[(size_t)i * n + k] * l[(size_t)j * n + k];
      s[i] = v;
    }
    if (!(s[j] > 0)) return false;
    const double d = sqrt(s[j]);
    l[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; ++i) l[(size_t)i * n + j] = s[i] / d;
  }
  return true;
}

// validate_dense_inv_metric (validate_dense_inv_metric.hpp:20-30) through
// Stan Math's check_pos_definite: finite, symmetric to 1e-8, positive pivots.
bool dense_metric_ok(const double* a, int n, std::vector<double>& l) {
  for (size_t k = 0; k < (size_t)n * n; ++k)
    if (!isfinite(a[k])) return false;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (fabs(a[(size_t)i * n + j] - a[(size_t)j * n + i]) > 1e-8) return false;
  return host_cholesky(a, n, l);
}

}  // namespace

int make_sampler_cfg(const gbnuts_model* m, const gbnuts_run_config* rc, int max_rows,
                     int out_cols, SamplerCfg* cfg_out, std::vector<std::string>* messages) {
  const int C = rc->num_chains;
  const int D = m->desc.D;
  if (C <= 0) return fail(GBNUTS_USAGE, "num_chains must be positive");
  if (rc->num_warmup < 0 || rc->num_samples < 0) return fail(GBNUTS_USAGE, "negative iterations");
  if (rc->num_thin < 1) return fail(GBNUTS_USAGE, "num_thin must be at least 1");
  // base_nuts::set_max_depth ignores non-positive depths (default 5)
  const int max_depth = rc->max_depth > 0 ? rc->max_depth : 5;
  if (max_depth > MAX_TREE_DEPTH) return fail(GBNUTS_USAGE, "max_depth above 16 is not supported");
  if (rc->metric != GBNUTS_METRIC_DIAG && rc->metric != GBNUTS_METRIC_DENSE)
    return fail(GBNUTS_USAGE, "metric must be GBNUTS_METRIC_DIAG or GBNUTS_METRIC_DENSE");
  if (rc->inv_metrics && rc->metric == GBNUTS_METRIC_DIAG) {
    for (size_t i = 0; i < (size_t)C * D; ++i)
      if (!isfinite(rc->inv_metrics[i]) || !(rc->inv_metrics[i] > 0))
        return fail(GBNUTS_CONFIG, "Inverse Euclidean metric not positive definite.");
  }
  if (rc->inv_metrics && rc->metric == GBNUTS_METRIC_DENSE) {
    std::vector<double> l;
    for (int c = 0; c < C; ++c)
      if (!dense_metric_ok(rc->inv_metrics + (size_t)c * D * D, D, l))
        return fail(GBNUTS_CONFIG, "Inverse Euclidean metric not positive definite.");
  }
  const int n_cols = 7 + D;
  const int warm_rows = rc->save_warmup ? (rc->num_warmup + rc->num_thin - 1) / rc->num_thin : 0;
  const int samp_rows = (rc->num_samples + rc->num_thin - 1) / rc->num_thin;
  const int need_rows = warm_rows + samp_rows;
  if (max_rows < need_rows || out_cols != n_cols)
    return fail(GBNUTS_USAGE, "output buffer too small (max_rows / n_cols)");

  SamplerCfg& cfg = *cfg_out;
  memset(&cfg, 0, sizeof(cfg));
  cfg.C = C;
  cfg.D = D;
  cfg.ld = (D + 3) & ~3;
  cfg.max_depth = max_depth;
  cfg.n_slots = SL_STACK + 6 * max_depth;
  cfg.adapt = rc->adapt ? 1 : 0;
  cfg.dense = rc->metric == GBNUTS_METRIC_DENSE ? 1 : 0;
  cfg.num_warmup = rc->num_warmup;
  cfg.num_samples = rc->num_samples;
  cfg.num_thin = rc->num_thin;
  cfg.save_warmup = rc->save_warmup ? 1 : 0;
  cfg.max_rows = max_rows;
  cfg.n_cols = n_cols;
  cfg.stepsize = rc->stepsize > 0 ? rc->stepsize : 0.1;  // set_nominal_stepsize ignores e <= 0
  cfg.jitter = (rc->stepsize_jitter > 0 && rc->stepsize_jitter < 1) ? rc->stepsize_jitter : 0.0;
  // stepsize_adaptation setters keep their defaults for invalid values
  cfg.delta = (rc->delta > 0 && rc->delta < 1) ? rc->delta : 0.5;
  cfg.gamma = rc->gamma > 0 ? rc->gamma : 0.05;
  cfg.kappa = rc->kappa > 0 ? rc->kappa : 0.75;
  cfg.t0 = rc->t0 > 0 ? rc->t0 : 10;
  cfg.init_radius = rc->init_radius;
  cfg.seed = rc->random_seed;
  cfg.init_chain_id = rc->init_chain_id;
  cfg.script_u = nullptr;
  cfg.script_z = nullptr;
  cfg.script_len = 0;
  cfg.idx_tau = m->desc.idx_tau;
  cfg.idx_sigma = m->desc.idx_sigma;
  WindowParams wp = window_params(rc->num_warmup, rc->init_buffer, rc->term_buffer, rc->window);
  if (rc->adapt) {
    cfg.wa_num_warmup = wp.num_warmup;
    cfg.wa_init_buffer = wp.init_buffer;
    cfg.wa_term_buffer = wp.term_buffer;
    cfg.wa_base_window = wp.base_window;
    cfg.wa_size0 = wp.size0;
    cfg.wa_next0 = wp.next0;
    if (messages) *messages = wp.messages;
  }
  return GBNUTS_OK;

}

extern "C" int gbnuts_sample_run(gbnuts_model* m, const gbnuts_run_config* rc,
                                 gbnuts_run_output* out, const gbnuts_callbacks* cb) {
  if (!m || !rc || !out) return fail(GBNUTS_USAGE, "bad arguments");
  if (!out->draws || !out->n_rows) return fail(GBNUTS_USAGE, "draws / n_rows buffers missing");
  const int C = rc->num_chains;
  const int D = m->desc.D;
  const int n_cols = 7 + D;
  SamplerCfg cfg;
  std::vector<std::string> wmsg;
  {
    int r = make_sampler_cfg(m, rc, out->max_rows, out->n_cols, &cfg, &wmsg);
    if (r) return r;
  }
  const int max_depth = cfg.max_depth;
  if (cb && cb->log)
    for (int c = 0; c < C; ++c)
      for (auto& msg : wmsg) cb->log(cb->ctx, GBNUTS_INFO, msg.c_str());

  cudaStream_t st = m->stream;
  DeviceRun dr;
  ChainState* d_states;
  ChainStack* d_stacks;
  double *d_vecs, *d_req, *d_draws, *d_diag = nullptr, *d_init, *d_inits = nullptr,
                                    *d_invm = nullptr;
  int *d_active, *d_done, *d_abort;
  GBN_CUDA_TRY(dr.alloc(&d_states, C));
  GBN_CUDA_TRY(dr.alloc(&d_stacks, C));
  GBN_CUDA_TRY(dr.alloc(&d_vecs, (size_t)C * cfg.n_slots * cfg.ld));
  GBN_CUDA_TRY(dr.alloc(&d_req, (size_t)C * cfg.ld));
  GBN_CUDA_TRY(dr.alloc(&d_active, C));
  GBN_CUDA_TRY(dr.alloc(&d_draws, (size_t)C * out->max_rows * n_cols));
  if (out->diagnostics) GBN_CUDA_TRY(dr.alloc(&d_diag, (size_t)C * out->max_rows * 3 * D));
  GBN_CUDA_TRY(dr.alloc(&d_init, (size_t)C * D));
  GBN_CUDA_TRY(dr.alloc(&d_done, 1));
  GBN_CUDA_TRY(dr.alloc(&d_abort, 1));
  if (rc->inits) {
    GBN_CUDA_TRY(dr.alloc(&d_inits, (size_t)C * D));
    GBN_CUDA_TRY(cudaMemcpyAsync(d_inits, rc->inits, (size_t)C * D * sizeof(double),
                                 cudaMemcpyHostToDevice, st));
  }
  if (g_draw_script.len > 0) {
    // scripted draws (test hook): every chain's uniform and normal streams
    const size_t n = (size_t)C * g_draw_script.len;
    double *d_su, *d_sz;
    GBN_CUDA_TRY(dr.alloc(&d_su, n));
    GBN_CUDA_TRY(dr.alloc(&d_sz, n));
    GBN_CUDA_TRY(cudaMemcpyAsync(d_su, g_draw_script.u, n * sizeof(double),
                                 cudaMemcpyHostToDevice, st));
    GBN_CUDA_TRY(cudaMemcpyAsync(d_sz, g_draw_script.z, n * sizeof(double),
                                 cudaMemcpyHostToDevice, st));
    cfg.script_u = d_su;
    cfg.script_z = d_sz;
    cfg.script_len = g_draw_script.len;
  }
  if (rc->inv_metrics && !cfg.dense) {
    GBN_CUDA_TRY(dr.alloc(&d_invm, (size_t)C * D));
    GBN_CUDA_TRY(cudaMemcpyAsync(d_invm, rc->inv_metrics, (size_t)C * D * sizeof(double),
                                 cudaMemcpyHostToDevice, st));
  }
  // dense_e: per chain A (the inverse metric), its Cholesky factor L and the
  // Welford M2, column-major; A and L from the given metric or the identity
  double* d_dense = nullptr;
  const size_t DD = (size_t)D * D;
  if (cfg.dense) {
    GBN_CUDA_TRY(dr.alloc(&d_dense, (size_t)C * 3 * DD));
    std::vector<double> h((size_t)2 * DD), l;
    for (int c = 0; c < C; ++c) {
      std::fill(h.begin(), h.end(), 0.0);
      if (rc->inv_metrics) {
        const double* a = rc->inv_metrics + (size_t)c * DD;
        host_cholesky(a, D, l);
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) {
            h[(size_t)j * D + i] = a[(size_t)i * D + j];
            h[DD + (size_t)j * D + i] = l[(size_t)i * D + j];
          }
      } else {
        for (int i = 0; i < D; ++i) h[(size_t)i * D + i] = h[DD + (size_t)i * D + i] = 1.0;
      }
      GBN_CUDA_TRY(cudaMemcpy(d_dense + (size_t)c * 3 * DD, h.data(), 2 * DD * sizeof(double),
                              cudaMemcpyHostToDevice));
      GBN_CUDA_TRY(cudaMemsetAsync(d_dense + (size_t)c * 3 * DD + 2 * DD, 0,
                                   DD * sizeof(double), st));
    }
  }
  GBN_CUDA_TRY(cudaMemsetAsync(d_done, 0, sizeof(int), st));
  GBN_CUDA_TRY(cudaMemsetAsync(d_abort, 0, sizeof(int), st));
  GBN_CUDA_TRY(cudaMemsetAsync(d_req, 0, (size_t)C * cfg.ld * sizeof(double), st));
  GBN_CUDA_TRY(cudaMemsetAsync(d_draws, 0, (size_t)C * out->max_rows * n_cols * sizeof(double), st));
  int prc = ensure_precision(m, rc->precision);
  if (prc) return prc;
  prc = prepare_workspace(m->desc, m->h_group_off.data(), C, rc->precision, m->ws);
  if (prc) return prc;
  const PartialsView pv{m->ws.partial, m->ws.NP, m->ws.S, m->ws.gz,
                        tct_dynamic(m->desc, rc->precision, C) ? m->ws.dyn : nullptr};

  int* h_done = nullptr;
  GBN_CUDA_TRY(cudaMallocHost(&h_done, sizeof(int)));
  struct RunGuard {
    int* pinned = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~RunGuard() {
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      if (pinned) cudaFreeHost(pinned);
    }
  } guard;
  guard.pinned = h_done;

  cudaEvent_t ev_begin, ev_end;
  GBN_CUDA_TRY(cudaEventCreate(&ev_begin));
  GBN_CUDA_TRY(cudaEventCreate(&ev_end));
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> grad_events;
  const size_t kMaxSamples = 512;

  launch_nuts_init(cfg, d_states, d_stacks, d_vecs, d_invm, d_active, st);
  GBN_CUDA_TRY(cudaGetLastError());
  GBN_CUDA_TRY(cudaEventRecord(ev_begin, st));
  auto wall0 = std::chrono::steady_clock::now();

  // The step kernel and (for the fp64 / fp32 forms with up to 16 chains per
  // block) the partial kernel run over one-entry fit tables: the same
  // launches a pool makes, so the fit's draws equal its draws in any pool.
  PoolFitDev h_fit;
  h_fit.cfg = cfg;
  h_fit.m = m->desc;
  h_fit.f = FitPtrs{d_states, d_stacks, d_vecs, d_req, pv, d_active, d_draws,
                    d_diag, d_init, d_inits, d_done, d_abort};
  h_fit.f.dense = d_dense;
  if (g_drain) {
    h_fit.f.h_rows = g_drain->rows;
    h_fit.f.h_diag = d_diag ? g_drain->diag : nullptr;
    h_fit.f.h_count = g_drain->count;
    h_fit.f.h_init = g_drain->init;
    h_fit.f.h_adapt = g_drain->adapt;
    h_fit.f.h_flag = g_drain->flag;
  }
  // the tensor-memory gradient kernel reads the request as packed words
  uint32_t* d_reqw = nullptr;
  struct WordsGuard {
    GradWorkspace* ws = nullptr;
    ~WordsGuard() {
      if (ws) ws->tc_words = nullptr;
    }
  } words_guard;
  if (is_tensor_precision(rc->precision) &&
      (rc->precision == GBNUTS_PREC_F16X3 ? m->desc.tc_xt16 : m->desc.tc_xt)) {
    GBN_CUDA_TRY(dr.alloc(&d_reqw, (size_t)C * tc::kThetaWords));
    h_fit.f.req_tc = d_reqw;
    h_fit.f.req_tc_f16 = rc->precision == GBNUTS_PREC_F16X3 ? 1 : 0;
    m->ws.tc_words = d_reqw;
    words_guard.ws = &m->ws;
  }
  std::vector<int2> h_cmap(C);
  for (int c = 0; c < C; ++c) h_cmap[c] = make_int2(0, c);
  PoolFitDev* d_fit;
  int2* d_cmap;
  GBN_CUDA_TRY(dr.alloc(&d_fit, 1));
  GBN_CUDA_TRY(dr.alloc(&d_cmap, C));
  GBN_CUDA_TRY(cudaMemcpyAsync(d_fit, &h_fit, sizeof(h_fit), cudaMemcpyHostToDevice, st));
  GBN_CUDA_TRY(cudaMemcpyAsync(d_cmap, h_cmap.data(), C * sizeof(int2), cudaMemcpyHostToDevice, st));
  const bool pool_partials = !is_tensor_precision(rc->precision);
  const int blk_chains = block_chains(m->desc.K, C);
  PoolGradFit* d_gfit = nullptr;
  PoolWorkItem* d_items = nullptr;
  int n_items = 0;
  size_t pool_smem = 0;
  if (pool_partials) {
    const PoolGradFit g{m->desc, d_req, cfg.ld, C, d_active, m->ws.split_rows, m->ws.partial,
                        m->ws.NP, m->ws.gz};
    const int rb = partial_tile_rows(m->desc.K, C, rc->precision);
    pool_smem = partial_smem(m->desc.K, C, rb, rc->precision);
    std::vector<PoolWorkItem> items;
    for (int s = 0; s < m->ws.S; ++s)
      for (int b = 0; b < (C + blk_chains - 1) / blk_chains; ++b)
        items.push_back(PoolWorkItem{0, s, b, rb});
    n_items = (int)items.size();
    GBN_CUDA_TRY(dr.alloc(&d_gfit, 1));
    GBN_CUDA_TRY(dr.alloc(&d_items, items.size()));
    GBN_CUDA_TRY(cudaMemcpyAsync(d_gfit, &g, sizeof(g), cudaMemcpyHostToDevice, st));
    GBN_CUDA_TRY(cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(PoolWorkItem),
                                 cudaMemcpyHostToDevice, st));
    // the host tables must outlive the copies
    GBN_CUDA_TRY(cudaStreamSynchronize(st));
  }

  // One step: every chain's state machine runs to its next gradient request,
  // then the gradient stage writes split partials the next step finalises.
  auto enqueue_step = [&](cudaEvent_t e0, cudaEvent_t e1) -> int {
    launch_nuts_step_pool(d_fit, d_cmap, C, team_warps(D), st);
    if (!pool_partials)
      return launch_partials(m->desc, rc->precision, d_req, cfg.ld, C, d_active, m->ws, st, e0,
                             e1);
    if (m->desc.off_z >= 0)
      GBN_CUDA_TRY(cudaMemsetAsync(m->ws.gz, 0, (size_t)C * m->desc.J * sizeof(double), st));
    if (e0) cudaEventRecord(e0, st);
    int r = launch_partials_pool(d_gfit, d_items, n_items, blk_chains, m->desc.x_dtype, rc->precision,
                                 pool_smem, st);
    if (e1) cudaEventRecord(e1, st);
    return r;
  };
  // Steps run in chunks of 32 captured once into a CUDA graph; every 16th
  // chunk runs eagerly with CUDA events around the gradient kernel (its live
  // launch time).  The first chunk is eager (it also sets kernel attributes).
  const int kChunk = 32;
  const int kTimedEvery = 16;
  bool use_graph = true;
  long long step = 0;
  const long long iters = (long long)rc->num_warmup + rc->num_samples;
  // upper bound on steps: every transition is at most 2^max_depth - 1 leapfrogs,
  // step-size searches are bounded by the 1e7 / 0 stops, 100 init tries.
  const long long max_steps = (iters + 2) * ((1LL << max_depth) + 200) + 1000;
  const int launches_per_step = 2 + (m->desc.off_z >= 0 ? 1 : 0);
  int status_rc = GBNUTS_OK;
  long long launches = 0;
  for (long long chunk_i = 0;; ++chunk_i) {
    const bool eager = !use_graph || (chunk_i % kTimedEvery) == 0;
    if (eager) {
      for (int k = 0; k < kChunk; ++k) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if ((k % 4) == 0 && grad_events.size() < kMaxSamples) {
          cudaEventCreate(&e0);
          cudaEventCreate(&e1);
          grad_events.emplace_back(e0, e1);
        }
        int r = enqueue_step(e0, e1);
        if (r) return r;
      }
    } else {
      if (!guard.exec) {
        int r = GBNUTS_OK;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
          for (int k = 0; k < kChunk && r == GBNUTS_OK; ++k) r = enqueue_step(nullptr, nullptr);
          cudaGraph_t g = nullptr;
          e = cudaStreamEndCapture(st, &g);
          guard.graph = g;
          if (e == cudaSuccess && r == GBNUTS_OK && g)
            e = cudaGraphInstantiate(&guard.exec, g, 0);
        }
        if (e != cudaSuccess || r != GBNUTS_OK || !guard.exec) {
          // capture unavailable: run every chunk eagerly
          cudaGetLastError();
          use_graph = false;
          for (int k = 0; k < kChunk; ++k) {
            int r2 = enqueue_step(nullptr, nullptr);
            if (r2) return r2;
          }
        }
      }
      if (use_graph) GBN_CUDA_TRY(cudaGraphLaunch(guard.exec, st));
    }
    step += kChunk;
    launches += (long long)kChunk * launches_per_step;
    GBN_CUDA_TRY(cudaMemcpyAsync(h_done, d_done, sizeof(int), cudaMemcpyDeviceToHost, st));
    GBN_CUDA_TRY(cudaStreamSynchronize(st));
    if (*h_done >= C) break;
    if (cb && cb->interrupt && cb->interrupt(cb->ctx)) {
      int one = 1;
      GBN_CUDA_TRY(cudaMemcpyAsync(d_abort, &one, sizeof(int), cudaMemcpyHostToDevice, st));
    }
    if (step > max_steps) {
      status_rc = fail(GBNUTS_SOFTWARE, "device run exceeded its step bound");
      break;
    }
  }
  GBN_CUDA_TRY(cudaEventRecord(ev_end, st));
  GBN_CUDA_TRY(cudaStreamSynchronize(st));
  auto wall1 = std::chrono::steady_clock::now();
  float total_ms = 0;
  cudaEventElapsedTime(&total_ms, ev_begin, ev_end);
  double grad_ms_sum = 0;
  int grad_n = 0;
  for (auto& pr : grad_events) {
    float t = 0;
    if (cudaEventElapsedTime(&t, pr.first, pr.second) == cudaSuccess) {
      grad_ms_sum += t;
      ++grad_n;
    }
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  cudaEventDestroy(ev_begin);
  cudaEventDestroy(ev_end);

  std::vector<ChainState> hs(C);
  GBN_CUDA_TRY(cudaMemcpy(hs.data(), d_states, C * sizeof(ChainState), cudaMemcpyDeviceToHost));
  if (out->ess || out->summary) {
    // convergence report on the device, before the draws leave it
    int w = 0, nr = out->max_rows;
    for (int c = 0; c < C; ++c) {
      w = std::max(w, hs[c].warm_rows);
      nr = std::min(nr, hs[c].rows);
    }
    const int re = fit_ess(d_draws, C, out->max_rows, n_cols, w, std::max(0, nr - w), out->ess,
                           out->summary, st);
    if (re) return re;
  }
  GBN_CUDA_TRY(cudaMemcpy(out->draws, d_draws, (size_t)C * out->max_rows * n_cols * sizeof(double),
                          cudaMemcpyDeviceToHost));
  if (out->diagnostics && d_diag)
    GBN_CUDA_TRY(cudaMemcpy(out->diagnostics, d_diag,
                            (size_t)C * out->max_rows * 3 * D * sizeof(double),
                            cudaMemcpyDeviceToHost));
  if (out->init)
    GBN_CUDA_TRY(cudaMemcpy(out->init, d_init, (size_t)C * D * sizeof(double),
                            cudaMemcpyDeviceToHost));
  if (out->inv_metric && cfg.dense) {
    std::vector<double> h(DD);
    for (int c = 0; c < C; ++c) {
      GBN_CUDA_TRY(cudaMemcpy(h.data(), d_dense + (size_t)c * 3 * DD, DD * sizeof(double),
                              cudaMemcpyDeviceToHost));
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j)
          out->inv_metric[(size_t)c * DD + (size_t)i * D + j] = h[(size_t)j * D + i];
    }
  } else if (out->inv_metric)
    GBN_CUDA_TRY(cudaMemcpy2D(out->inv_metric, D * sizeof(double),
                              d_vecs + (size_t)SL_INVM * cfg.ld,
                              (size_t)cfg.n_slots * cfg.ld * sizeof(double), D * sizeof(double),
                              C, cudaMemcpyDeviceToHost));
  const double wall_s = std::chrono::duration<double>(wall1 - wall0).count();
  for (int c = 0; c < C; ++c) {
    out->n_rows[c] = hs[c].rows;
    if (out->n_warmup_rows) out->n_warmup_rows[c] = hs[c].warm_rows;
    if (out->status) out->status[c] = hs[c].status;
    if (out->stepsize) out->stepsize[c] = hs[c].nom_eps;
    if (out->n_grad) out->n_grad[c] = hs[c].n_grad;
    if (out->seconds) {
      // each chain's warmup share of the run, by its gradient count
      const double frac = (hs[c].warm_end_ngrad >= 0 && hs[c].n_grad > 0)
                              ? (double)hs[c].warm_end_ngrad / (double)hs[c].n_grad
                              : 0.0;
      out->seconds[2 * c] = wall_s * frac;
      out->seconds[2 * c + 1] = wall_s * (1.0 - frac);
    }
  }
  if (status_rc == GBNUTS_OK) status_rc = check_device_error(m->ws);
  out->total_ms = total_ms;
  out->grad_ms = grad_n ? grad_ms_sum / grad_n : 0.0;
  out->steps = step;
  out->kernel_launches = launches;
  return status_rc;
}

// ------------------------------------------------------------------ services
namespace {

std::string fmt(double v) {
  std::ostringstream s;
  s << v;
  return s.str();
}

void emit_msg(const gbnuts_callbacks* cb, int c, int w, const std::string& s) {
  if (cb && cb->write_message) cb->write_message(cb->ctx, c, w, s.c_str());
}
void emit_blank(const gbnuts_callbacks* cb, int c, int w) {
  if (cb && cb->write_blank) cb->write_blank(cb->ctx, c, w);
}
void emit_log(const gbnuts_callbacks* cb, int level, const std::string& s) {
  if (cb && cb->log) cb->log(cb->ctx, level, s.c_str());
}
void emit_names(const gbnuts_callbacks* cb, int c, int w, const std::vector<std::string>& v) {
  if (!cb || !cb->write_names) return;
  std::vector<const char*> p;
  for (auto& s : v) p.push_back(s.c_str());
  cb->write_names(cb->ctx, c, w, p.data(), (int)p.size());
}
void emit_values(const gbnuts_callbacks* cb, int c, int w, const double* v, int n) {
  if (cb && cb->write_values) cb->write_values(cb->ctx, c, w, v, n);
}

// mcmc_writer::write_timing (mcmc_writer.hpp:198-218) to one writer
void write_timing(const gbnuts_callbacks* cb, int c, int w, double warm, double samp) {
  const std::string title(" Elapsed Time: ");
  emit_blank(cb, c, w);
  emit_msg(cb, c, w, title + fmt(warm) + " seconds (Warm-up)");
  emit_msg(cb, c, w, std::string(title.size(), ' ') + fmt(samp) + " seconds (Sampling)");
  emit_msg(cb, c, w, std::string(title.size(), ' ') + fmt(warm + samp) + " seconds (Total)");
  emit_blank(cb, c, w);
}

// What a chain's writers have received so far: the host drain writes during
// the run, write_run completes the chain after it.
struct ChainEmit {
  bool init = false;   // init values
  bool names = false;  // header names
  int rows = 0;        // rows
  bool adapt = false;  // adaptation block
};

int write_run(const gbnuts_model* m, const gbnuts_run_config& rc, const gbnuts_run_output& o,
              const gbnuts_callbacks* cb, const std::vector<ChainEmit>* prior = nullptr);

// The service's writer protocol pieces shared by the drain and write_run.
struct WriterNames {
  std::vector<std::string> sample, diagnostic;
  explicit WriterNames(const ModelDesc& desc) {
    std::vector<std::string> cnames, unames;
    host_names(desc, true, cnames);
    host_names(desc, false, unames);
    const std::vector<std::string> sn = {"lp__", "accept_stat__", "stepsize__", "treedepth__",
                                         "n_leapfrog__", "divergent__", "energy__"};
    sample = sn;
    sample.insert(sample.end(), cnames.begin(), cnames.end());
    diagnostic = sn;
    for (auto& s : unames) diagnostic.push_back(s);
    for (auto& s : unames) diagnostic.push_back("p_" + s);
    for (auto& s : unames) diagnostic.push_back("g_" + s);
  }
};

// One row to the sample writer (and, with diag, the diagnostic writer: the
// sampler columns, then q, p, g).
void emit_row(const gbnuts_callbacks* cb, int c, const double* row, int n_cols,
              const double* diag, int D, std::vector<double>& drow) {
  emit_values(cb, c, GBNUTS_SAMPLE_WRITER, row, n_cols);
  if (diag) {
    drow.resize(7 + 3 * D);
    memcpy(drow.data(), row, 7 * sizeof(double));
    memcpy(drow.data() + 7, diag, 3 * D * sizeof(double));
    emit_values(cb, c, GBNUTS_DIAGNOSTIC_WRITER, drow.data(), 7 + 3 * D);
  }
}

// mcmc_writer::write_adapt_finish + base_hmc::write_sampler_state; invm
// row-major (D values for diag_e, D x D for dense_e).
void emit_adapt_block(const gbnuts_callbacks* cb, int c, const gbnuts_run_config& rc, int D,
                      double eps, const double* invm) {
  emit_msg(cb, c, GBNUTS_SAMPLE_WRITER, "Adaptation terminated");
  emit_msg(cb, c, GBNUTS_SAMPLE_WRITER, "Step size = " + fmt(eps));
  if (rc.metric == GBNUTS_METRIC_DENSE) {
    // dense_e_point::write_metric (dense_e_point.hpp:35-48)
    emit_msg(cb, c, GBNUTS_SAMPLE_WRITER, "Elements of inverse mass matrix:");
    if (D == 0) emit_msg(cb, c, GBNUTS_SAMPLE_WRITER, "");
    for (int i = 0; i < D; ++i) {
      std::ostringstream s;
      for (int j = 0; j < D; ++j) s << (j ? ", " : "") << invm[(size_t)i * D + j];
      emit_msg(cb, c, GBNUTS_SAMPLE_WRITER, s.str());
    }
    if (rc.adapt && cb && cb->write_metric) cb->write_metric(cb->ctx, c, eps, "dense_e", invm, D * D);
  } else {
    emit_msg(cb, c, GBNUTS_SAMPLE_WRITER, "Diagonal elements of inverse mass matrix:");
    std::ostringstream s;
    for (int d = 0; d < D; ++d) s << (d ? ", " : "") << invm[d];
    emit_msg(cb, c, GBNUTS_SAMPLE_WRITER, s.str());
    if (rc.adapt && cb && cb->write_metric) cb->write_metric(cb->ctx, c, eps, "diag_e", invm, D);
  }
}

// The service's host drain: the step kernel also writes every row, the init
// values and the end-of-warmup adaptation record into mapped host memory
// (DrainPtrs), each followed by a count or flag; host threads poll those and
// pass what has arrived to the writer callbacks while the device run goes on
// (chain c's calls in order, on thread c mod n).  Nothing is written until
// every chain has initialised (a failed initialisation reports only errors,
// as the reference's set-up does).  write_run completes each chain after the
// run from where the drain stopped.
class HostDrain {
 public:
  HostDrain(const gbnuts_model* m, const gbnuts_run_config& rc, const gbnuts_callbacks* cb,
            int max_rows, bool diag)
      : m_(m), rc_(rc), cb_(cb), C_(rc.num_chains), D_(m->desc.D), n_cols_(7 + m->desc.D),
        max_rows_(max_rows), names_(m->desc), emit_(rc.num_chains) {
    const int M = rc.metric == GBNUTS_METRIC_DENSE ? D_ * D_ : D_;
    adapt_stride_ = 1 + M;
    bytes_rows_ = (size_t)C_ * max_rows_ * n_cols_ * sizeof(double);
    bytes_diag_ = diag ? (size_t)C_ * max_rows_ * 3 * D_ * sizeof(double) : 0;
    const size_t bytes = bytes_rows_ + bytes_diag_ + (size_t)C_ * D_ * sizeof(double) +
                         (size_t)C_ * adapt_stride_ * sizeof(double) + (size_t)3 * C_ * sizeof(int);
    if (cudaHostAlloc(&base_, bytes, cudaHostAllocMapped) != cudaSuccess) {
      cudaGetLastError();
      base_ = nullptr;
      return;
    }
    char* p = static_cast<char*>(base_);
    rows_ = reinterpret_cast<double*>(p);
    p += bytes_rows_;
    diag_ = diag ? reinterpret_cast<double*>(p) : nullptr;
    p += bytes_diag_;
    init_ = reinterpret_cast<double*>(p);
    p += (size_t)C_ * D_ * sizeof(double);
    adapt_ = reinterpret_cast<double*>(p);
    p += (size_t)C_ * adapt_stride_ * sizeof(double);
    count_ = reinterpret_cast<int*>(p);
    flag_ = count_ + C_;
    memset(count_, 0, (size_t)3 * C_ * sizeof(int));
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, base_, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaFreeHost(base_);
      base_ = nullptr;
      return;
    }
    const ptrdiff_t off = static_cast<char*>(d) - static_cast<char*>(base_);
    auto dev = [&](void* h) { return static_cast<char*>(h) + off; };
    ptrs_.rows = reinterpret_cast<double*>(dev(rows_));
    ptrs_.diag = diag_ ? reinterpret_cast<double*>(dev(diag_)) : nullptr;
    ptrs_.count = reinterpret_cast<int*>(dev(count_));
    ptrs_.init = reinterpret_cast<double*>(dev(init_));
    ptrs_.adapt = reinterpret_cast<double*>(dev(adapt_));
    ptrs_.flag = reinterpret_cast<int*>(dev(flag_));
  }
  ~HostDrain() {
    stop();
    if (base_) cudaFreeHost(base_);
  }
  bool ok() const { return base_ != nullptr; }
  const DrainPtrs* ptrs() const { return &ptrs_; }

  void start() {
    const int nt = (cb_ && cb_->chains_concurrent)
                       ? std::min(C_, std::max(1, (int)std::thread::hardware_concurrency()))
                       : 1;
    for (int t = 0; t < nt; ++t)
      threads_.emplace_back([this, t, nt] {
        std::vector<double> drow;
        while (!stop_.load(std::memory_order_acquire)) {
          if (gate()) {
            for (int c = t; c < C_; c += nt) {
              try {
                pump(c, drow);
              } catch (...) {
              }
            }
          }
          std::this_thread::sleep_for(std::chrono::microseconds(500));
        }
      });
  }
  void stop() {
    stop_.store(true, std::memory_order_release);
    for (auto& t : threads_) t.join();
    threads_.clear();
  }
  const std::vector<ChainEmit>& emitted() const { return emit_; }

 private:
  int load(const int* p) const { return *reinterpret_cast<const volatile int*>(p); }
  // open once every chain has written its init values
  bool gate() {
    if (open_.load(std::memory_order_acquire)) return true;
    for (int c = 0; c < C_; ++c)
      if (!load(flag_ + 2 * c)) return false;
    std::atomic_thread_fence(std::memory_order_acquire);
    open_.store(true, std::memory_order_release);
    return true;
  }
  void pump(int c, std::vector<double>& drow) {
    ChainEmit& e = emit_[c];
    if (!e.init) {
      emit_values(cb_, c, GBNUTS_INIT_WRITER, init_ + (size_t)c * D_, D_);
      e.init = true;
    }
    const int count = std::min(load(count_ + c), max_rows_);
    std::atomic_thread_fence(std::memory_order_acquire);
    if (count <= e.rows) return;
    if (!e.names) {
      emit_names(cb_, c, GBNUTS_SAMPLE_WRITER, names_.sample);
      emit_names(cb_, c, GBNUTS_DIAGNOSTIC_WRITER, names_.diagnostic);
      e.names = true;
    }
    const int thin = std::max(1, rc_.num_thin);
    const int n_warm = rc_.save_warmup ? (rc_.num_warmup + thin - 1) / thin : 0;
    while (e.rows < count) {
      if (e.rows == n_warm && !e.adapt) {
        if (!load(flag_ + 2 * c + 1)) return;
        std::atomic_thread_fence(std::memory_order_acquire);
        const double* rec = adapt_ + (size_t)c * adapt_stride_;
        if (rc_.metric == GBNUTS_METRIC_DENSE) {
          // the record is column-major; the block prints it row-major
          std::vector<double> a((size_t)D_ * D_);
          for (int i = 0; i < D_; ++i)
            for (int j = 0; j < D_; ++j) a[(size_t)i * D_ + j] = rec[1 + (size_t)j * D_ + i];
          emit_adapt_block(cb_, c, rc_, D_, rec[0], a.data());
        } else {
          emit_adapt_block(cb_, c, rc_, D_, rec[0], rec + 1);
        }
        e.adapt = true;
      }
      const size_t ri = (size_t)c * max_rows_ + e.rows;
      emit_row(cb_, c, rows_ + ri * n_cols_, n_cols_, diag_ ? diag_ + ri * 3 * D_ : nullptr, D_,
               drow);
      ++e.rows;
    }
  }

  const gbnuts_model* m_;
  gbnuts_run_config rc_;
  const gbnuts_callbacks* cb_;
  int C_, D_, n_cols_, max_rows_, adapt_stride_ = 0;
  WriterNames names_;
  std::vector<ChainEmit> emit_;
  void* base_ = nullptr;
  size_t bytes_rows_ = 0, bytes_diag_ = 0;
  double *rows_ = nullptr, *diag_ = nullptr, *init_ = nullptr, *adapt_ = nullptr;
  int *count_ = nullptr, *flag_ = nullptr;
  DrainPtrs ptrs_{};
  std::vector<std::thread> threads_;
  std::atomic<bool> stop_{false}, open_{false};
};

int run_service(gbnuts_model* m, gbnuts_run_config rc, const gbnuts_callbacks* cb) {
  const int C = rc.num_chains, D = m ? m->desc.D : 0;
  if (!m || C <= 0) return fail(GBNUTS_USAGE, "bad arguments");
  const int n_cols = 7 + D;
  const int thin = std::max(1, rc.num_thin);
  const int rows = (rc.save_warmup ? (rc.num_warmup + thin - 1) / thin : 0) +
                   (rc.num_samples + thin - 1) / thin;
  const bool diag = cb && cb->want_diagnostics;
  std::vector<double> draws((size_t)C * std::max(rows, 1) * n_cols), dg;
  if (diag) dg.resize((size_t)C * std::max(rows, 1) * 3 * D);
  std::vector<int> n_rows(C), n_warm(C), status(C);
  std::vector<double> eps(C), invm((size_t)C * D * (rc.metric == GBNUTS_METRIC_DENSE ? D : 1)),
      init((size_t)C * D), secs(2 * C);
  std::vector<long long> ngrad(C);
  gbnuts_run_output o;
  memset(&o, 0, sizeof(o));
  o.max_rows = std::max(rows, 1);
  o.n_cols = n_cols;
  o.draws = draws.data();
  o.diagnostics = diag ? dg.data() : nullptr;
  o.n_rows = n_rows.data();
  o.n_warmup_rows = n_warm.data();
  o.status = status.data();
  o.stepsize = eps.data();
  o.inv_metric = invm.data();
  o.init = init.data();
  o.n_grad = ngrad.data();
  o.seconds = secs.data();
  // rows reach the writers while the run goes on (when mapped host memory
  // can be had; otherwise all of them after it)
  HostDrain drain(m, rc, cb, o.max_rows, diag);
  if (drain.ok()) {
    g_drain = drain.ptrs();
    drain.start();
  }
  int r = gbnuts_sample_run(m, &rc, &o, cb);
  g_drain = nullptr;
  drain.stop();
  if (r == GBNUTS_CONFIG) {
    emit_log(cb, GBNUTS_ERROR, last_error());
    return r;
  }
  if (r) return r;
  // set-up failures are reported before any chain runs (hmc_nuts_diag_e_adapt.hpp:359-385)
  for (int c = 0; c < C; ++c) {
    if (status[c] == GBNUTS_CHAIN_INIT_FAILED) {
      if (rc.init_radius != 0.0 && !rc.inits) {
        emit_log(cb, GBNUTS_INFO, "");
        emit_log(cb, GBNUTS_ERROR, "Initialization between (-" + fmt(rc.init_radius) + ", " +
                                       fmt(rc.init_radius) + ") failed after 100 attempts. ");
        emit_log(cb, GBNUTS_ERROR,
                 " Try specifying initial values, reducing ranges of constrained values, "
                 "or reparameterizing the model.");
      }
      emit_log(cb, GBNUTS_ERROR, "Initialization failed.");
      return GBNUTS_CONFIG;
    }
  }
  return write_run(m, rc, o, cb, drain.ok() ? &drain.emitted() : nullptr);
}

// Writes a finished run through the writer callbacks in the service protocol
// (mcmc_writer.hpp:63-259, run_adaptive_sampler.hpp:46-103): per chain the
// init values, the names, warmup rows, the adaptation block, sampling rows and
// the timing block, with the reference's messages for failed chains.
int write_run(const gbnuts_model* m, const gbnuts_run_config& rc, const gbnuts_run_output& o,
              const gbnuts_callbacks* cb, const std::vector<ChainEmit>* prior) {
  const int C = rc.num_chains, D = m->desc.D, n_cols = 7 + D;
  const bool diag = cb && cb->want_diagnostics && o.diagnostics;
  const int* status = o.status;
  const int* n_rows = o.n_rows;
  const int* n_warm = o.n_warmup_rows;
  const double* eps = o.stepsize;
  const double* invm = o.inv_metric;
  const double* init = o.init;
  const double* secs = o.seconds;
  const WriterNames names(m->desc);
  // one chain's rows and messages, in the reference's order, from where the
  // drain (if any) stopped; chains touch only their own writers
  auto emit_chain = [&](int c) -> int {
    const ChainEmit e = prior ? (*prior)[c] : ChainEmit();
    std::vector<double> drow(7 + 3 * D);
    if (!e.init) emit_values(cb, c, GBNUTS_INIT_WRITER, init + (size_t)c * D, D);
    if (status[c] == GBNUTS_CHAIN_STEPSIZE_INIT_FAILED) {
      // run_adaptive_sampler.hpp:61-68
      emit_log(cb, GBNUTS_ERROR, "Exception initializing step size.");
      emit_log(cb, GBNUTS_ERROR, "Posterior is improper. Please check your model.");
      return GBNUTS_OK;
    }
    if (!e.names) {
      emit_names(cb, c, GBNUTS_SAMPLE_WRITER, names.sample);
      emit_names(cb, c, GBNUTS_DIAGNOSTIC_WRITER, names.diagnostic);
    }
    const double* base = o.draws + (size_t)c * o.max_rows * n_cols;
    auto write_rows = [&](int from, int to) {
      for (int i = from; i < to; ++i)
        emit_row(cb, c, base + (size_t)i * n_cols, n_cols,
                 diag ? o.diagnostics + ((size_t)c * o.max_rows + i) * 3 * D : nullptr, D, drow);
    };
    write_rows(std::min(e.rows, n_warm[c]), n_warm[c]);
    const bool complete = status[c] == GBNUTS_CHAIN_OK;
    if (!e.adapt && (complete || n_rows[c] > n_warm[c]))
      emit_adapt_block(cb, c, rc, D, eps[c],
                       invm + (size_t)c * D * (rc.metric == GBNUTS_METRIC_DENSE ? D : 1));
    write_rows(std::max(e.rows, n_warm[c]), n_rows[c]);
    if (status[c] == GBNUTS_CHAIN_OK) {
      write_timing(cb, c, GBNUTS_SAMPLE_WRITER, secs[2 * c], secs[2 * c + 1]);
      write_timing(cb, c, GBNUTS_DIAGNOSTIC_WRITER, secs[2 * c], secs[2 * c + 1]);
      const std::string title(" Elapsed Time: ");
      emit_log(cb, GBNUTS_INFO, "");
      emit_log(cb, GBNUTS_INFO, title + fmt(secs[2 * c]) + " seconds (Warm-up)");
      emit_log(cb, GBNUTS_INFO,
               std::string(title.size(), ' ') + fmt(secs[2 * c + 1]) + " seconds (Sampling)");
      emit_log(cb, GBNUTS_INFO, std::string(title.size(), ' ') +
                                    fmt(secs[2 * c] + secs[2 * c + 1]) + " seconds (Total)");
      emit_log(cb, GBNUTS_INFO, "");
    } else if (status[c] == GBNUTS_CHAIN_STEPSIZE_FAILED ||
               status[c] == GBNUTS_CHAIN_METRIC_OVERFLOW ||
               status[c] == GBNUTS_CHAIN_INTERRUPTED) {
      if (status[c] == GBNUTS_CHAIN_METRIC_OVERFLOW)
        emit_log(cb, GBNUTS_ERROR,
                 "Numerical overflow in metric adaptation. This occurs when the sampler "
                 "encounters extreme values on the unconstrained space; this may happen when "
                 "the posterior density function is too wide or improper. There may be "
                 "problems with your model specification.");
      else if (status[c] == GBNUTS_CHAIN_STEPSIZE_FAILED)
        emit_log(cb, GBNUTS_ERROR, "Posterior is improper. Please check your model.");
      else
        emit_log(cb, GBNUTS_ERROR, "Sampling interrupted.");
      return GBNUTS_SOFTWARE;
    }
    return GBNUTS_OK;
  };
  std::vector<int> codes(C, GBNUTS_OK);
  const int nt = (cb && cb->chains_concurrent)
                     ? std::min(C, std::max(1, (int)std::thread::hardware_concurrency()))
                     : 1;
  if (nt > 1) {
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
      pool.emplace_back([&] {
        for (int c; (c = next.fetch_add(1)) < C;) {
          try {
            codes[c] = emit_chain(c);
          } catch (...) {
            codes[c] = GBNUTS_SOFTWARE;
          }
        }
      });
    for (auto& t : pool) t.join();
  } else {
    for (int c = 0; c < C; ++c) codes[c] = emit_chain(c);
  }
  int code = GBNUTS_OK;
  for (int c = 0; c < C; ++c)
    if (codes[c] != GBNUTS_OK) code = codes[c];
  return code;
}

}  // namespace

static int nuts_adapt_service(int metric,
    gbnuts_model* m, int num_chains, const double* inits, const double* inv_metrics,
    unsigned random_seed, unsigned init_chain_id, double init_radius, int num_warmup,
    int num_samples, int num_thin, int save_warmup, int refresh, double stepsize,
    double stepsize_jitter, int max_depth, double delta, double gamma, double kappa, double t0,
    unsigned init_buffer, unsigned term_buffer, unsigned window, int precision,
    const gbnuts_callbacks* cb) {
  (void)refresh;
  gbnuts_run_config rc;
  memset(&rc, 0, sizeof(rc));
  rc.num_chains = num_chains;
  rc.adapt = 1;
  rc.num_warmup = num_warmup;
  rc.num_samples = num_samples;
  rc.num_thin = num_thin;
  rc.save_warmup = save_warmup;
  rc.stepsize = stepsize;
  rc.stepsize_jitter = stepsize_jitter;
  rc.max_depth = max_depth;
  rc.delta = delta;
  rc.gamma = gamma;
  rc.kappa = kappa;
  rc.t0 = t0;
  rc.init_buffer = init_buffer;
  rc.term_buffer = term_buffer;
  rc.window = window;
  rc.init_radius = init_radius;
  rc.random_seed = random_seed;
  rc.init_chain_id = init_chain_id;
  rc.precision = precision;
  rc.inits = inits;
  rc.inv_metrics = inv_metrics;
  rc.metric = metric;
  return run_service(m, rc, cb);
}

extern "C" int gbnuts_hmc_nuts_diag_e_adapt(
    gbnuts_model* m, int num_chains, const double* inits, const double* inv_metrics,
    unsigned random_seed, unsigned init_chain_id, double init_radius, int num_warmup,
    int num_samples, int num_thin, int save_warmup, int refresh, double stepsize,
    double stepsize_jitter, int max_depth, double delta, double gamma, double kappa, double t0,
    unsigned init_buffer, unsigned term_buffer, unsigned window, int precision,
    const gbnuts_callbacks* cb) {
  return nuts_adapt_service(GBNUTS_METRIC_DIAG, m, num_chains, inits, inv_metrics, random_seed,
                            init_chain_id, init_radius, num_warmup, num_samples, num_thin,
                            save_warmup, refresh, stepsize, stepsize_jitter, max_depth, delta,
                            gamma, kappa, t0, init_buffer, term_buffer, window, precision, cb);
}

extern "C" int gbnuts_hmc_nuts_dense_e_adapt(
    gbnuts_model* m, int num_chains, const double* inits, const double* inv_metrics,
    unsigned random_seed, unsigned init_chain_id, double init_radius, int num_warmup,
    int num_samples, int num_thin, int save_warmup, int refresh, double stepsize,
    double stepsize_jitter, int max_depth, double delta, double gamma, double kappa, double t0,
    unsigned init_buffer, unsigned term_buffer, unsigned window, int precision,
    const gbnuts_callbacks* cb) {
  return nuts_adapt_service(GBNUTS_METRIC_DENSE, m, num_chains, inits, inv_metrics, random_seed,
                            init_chain_id, init_radius, num_warmup, num_samples, num_thin,
                            save_warmup, refresh, stepsize, stepsize_jitter, max_depth, delta,
                            gamma, kappa, t0, init_buffer, term_buffer, window, precision, cb);
}

static int nuts_service(int metric, gbnuts_model* m, int num_chains, const double* inits,
                                      const double* inv_metrics, unsigned random_seed,
                                      unsigned init_chain_id, double init_radius,
                                      int num_warmup, int num_samples, int num_thin,
                                      int save_warmup, int refresh, double stepsize,
                                      double stepsize_jitter, int max_depth, int precision,
                                      const gbnuts_callbacks* cb) {
  (void)refresh;
  gbnuts_run_config rc;
  memset(&rc, 0, sizeof(rc));
  rc.num_chains = num_chains;
  rc.adapt = 0;
  rc.num_warmup = num_warmup;
  rc.num_samples = num_samples;
  rc.num_thin = num_thin;
  rc.save_warmup = save_warmup;
  rc.stepsize = stepsize;
  rc.stepsize_jitter = stepsize_jitter;
  rc.max_depth = max_depth;
  rc.init_radius = init_radius;
  rc.random_seed = random_seed;
  rc.init_chain_id = init_chain_id;
  rc.precision = precision;
  rc.inits = inits;
  rc.inv_metrics = inv_metrics;
  rc.metric = metric;
  return run_service(m, rc, cb);
}

extern "C" int gbnuts_hmc_nuts_diag_e(gbnuts_model* m, int num_chains, const double* inits,
                                      const double* inv_metrics, unsigned random_seed,
                                      unsigned init_chain_id, double init_radius,
                                      int num_warmup, int num_samples, int num_thin,
                                      int save_warmup, int refresh, double stepsize,
                                      double stepsize_jitter, int max_depth, int precision,
                                      const gbnuts_callbacks* cb) {
  return nuts_service(GBNUTS_METRIC_DIAG, m, num_chains, inits, inv_metrics, random_seed,
                      init_chain_id, init_radius, num_warmup, num_samples, num_thin, save_warmup,
                      refresh, stepsize, stepsize_jitter, max_depth, precision, cb);
}

extern "C" int gbnuts_hmc_nuts_dense_e(gbnuts_model* m, int num_chains, const double* inits,
                                      const double* inv_metrics, unsigned random_seed,
                                      unsigned init_chain_id, double init_radius,
                                      int num_warmup, int num_samples, int num_thin,
                                      int save_warmup, int refresh, double stepsize,
                                      double stepsize_jitter, int max_depth, int precision,
                                      const gbnuts_callbacks* cb) {
  return nuts_service(GBNUTS_METRIC_DENSE, m, num_chains, inits, inv_metrics, random_seed,
                      init_chain_id, init_radius, num_warmup, num_samples, num_thin, save_warmup,
                      refresh, stepsize, stepsize_jitter, max_depth, precision, cb);
}

extern "C" int gbnuts_write_run(const gbnuts_model* m, const gbnuts_run_config* rc,
                                const gbnuts_run_output* out, const gbnuts_callbacks* cb) {
  using namespace gbn;
  if (!m || !rc || !out || rc->num_chains <= 0 || !out->draws || !out->n_rows ||
      !out->n_warmup_rows || !out->status || !out->stepsize || !out->inv_metric || !out->init ||
      !out->seconds || out->n_cols != 7 + m->desc.D || out->max_rows <= 0) {
    set_last_error("gbnuts_write_run: bad arguments");
    return GBNUTS_USAGE;
  }
  for (int c = 0; c < rc->num_chains; ++c)
    if (out->n_rows[c] < 0 || out->n_rows[c] > out->max_rows || out->n_warmup_rows[c] < 0 ||
        out->n_warmup_rows[c] > out->n_rows[c]) {
      set_last_error("gbnuts_write_run: row counts outside the output");
      return GBNUTS_USAGE;
    }
  try {
    return write_run(m, *rc, *out, cb);
  } catch (const std::exception& e) {
    set_last_error(std::string("gbnuts_write_run: ") + e.what());
    return GBNUTS_SOFTWARE;
  }
}
