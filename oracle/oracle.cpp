// TEST INFRASTRUCTURE: the CPU oracle for the gbnuts hot path.
//
// A plain C++17 FP64 restatement of the reference's NUTS (diag_e, adaptive)
// sampling path, used only by tests/, the smoke check and bench.py's CPU
// baseline leg.  Nothing in the product links, imports or calls this file.
//
// It follows, function by function (paths relative to the stan-dev/stan tree):
//   src/stan/mcmc/hmc/nuts/base_nuts.hpp:78-352         transition, build_tree
//   src/stan/mcmc/hmc/nuts/adapt_diag_e_nuts.hpp:25-48  adaptive transition
//   src/stan/mcmc/hmc/base_hmc.hpp:93-200               init_stepsize, sample_stepsize
//   src/stan/mcmc/hmc/hamiltonians/diag_e_metric.hpp:20-50, base_hamiltonian.hpp:48-70
//   src/stan/mcmc/hmc/integrators/expl_leapfrog.hpp:16-32, base_leapfrog.hpp:17-22
//   src/stan/mcmc/stepsize_adaptation.hpp:13-73, windowed_adaptation.hpp:14-110,
//   src/stan/mcmc/var_adaptation.hpp:17-46
//   src/stan/services/util/initialize.hpp:68-227, run_adaptive_sampler.hpp:46-103,
//   src/stan/services/util/run_sampler.hpp, generate_transitions.hpp:42-77,
//   src/stan/services/sample/hmc_nuts_diag_e_adapt.hpp:57-112, hmc_nuts_diag_e.hpp:48-100
// The build_tree recursion is kept recursive here (the GPU path is iterative),
// so agreement between the two is a check of the iterative formulation.
//
// Third-party arithmetic that lives outside the reference tree is restated from
// its definition: stan::math::log_sum_exp / log1p_exp (call sites
// base_nuts.hpp:172,265,323-324), stan::math::welford_var_estimator
// (var_adaptation.hpp:49), and the log densities (bernoulli_logit, poisson_log,
// normal) of Stan Math.  Boost mixmax / normal_distribution are replaced by the
// gbnuts draw stream (include/gbnuts_draw_stream.h), consumed in the same order
// as the reference consumes its RNG.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off, so elementwise leapfrog
// updates round exactly as the GPU path's explicit _rn operations do).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../include/gbnuts_draw_stream.h"

namespace oracle {

using Vec = std::vector<double>;
static const double INF = std::numeric_limits<double>::infinity();
static const double LOG_SQRT_2PI = 0.91893853320467274178032973640562;

// ---------------------------------------------------------------- math
// stan::math::log1p_exp: log(1 + exp(a)) without overflow.
static double log1p_exp(double a) {
  if (a > 0.0) return a + std::log1p(std::exp(-a));
  return std::log1p(std::exp(a));
}

// stan::math::log_sum_exp(a, b) for scalars.
static double log_sum_exp(double a, double b) {
  if (a == -INF) return b;
  if (a == INF && b == INF) return INF;
  if (a > b) return a + log1p_exp(b - a);
  return b + log1p_exp(a - b);
}

static double inv_logit(double x) {
  if (x >= 0) return 1.0 / (1.0 + std::exp(-x));
  double e = std::exp(x);
  return e / (1.0 + e);
}

static double dot(const Vec& a, const Vec& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

// Neumaier compensated summation, used for every sum over data rows.
struct CSum {
  double s = 0.0, c = 0.0;
  void add(double x) {
    double t = s + x;
    if (std::fabs(s) >= std::fabs(x))
      c += (s - t) + x;
    else
      c += (x - t) + s;
    s = t;
  }
  double value() const { return s + c; }
};

// ---------------------------------------------------------------- models
enum ModelKind { LOGISTIC = 1, POISSON = 2, HIER_NORMAL = 3, HIER_LOGISTIC = 4 };

struct Model {
  int kind = LOGISTIC;
  int N = 0, K = 0, J = 0, D = 0;
  int intercept = 1;
  Vec X;                  // N*K row-major
  Vec y;                  // N
  std::vector<int> group; // N, 0-based group of each row
  Vec hp;                 // hyperparameters (prior scales)
  int compensated = 1;    // Neumaier sums over rows (GLMs)

  void finalize() {
    switch (kind) {
      case LOGISTIC: D = K + (intercept ? 1 : 0); break;
      case POISSON: D = K + (intercept ? 1 : 0); break;
      case HIER_NORMAL: D = 3 + J + K; break;
      case HIER_LOGISTIC: D = 2 + J + K; break;
      default: throw std::invalid_argument("unknown model kind");
    }
  }

  double hpv(int i, double dflt) const {
    return (i < (int)hp.size()) ? hp[i] : dflt;
  }

  // log density (and gradient when grad != nullptr) on the unconstrained
  // scale, with Stan's propto / jacobian semantics.
  double eval(const double* th, double* grad, bool propto, bool jacobian) const {
    switch (kind) {
      case LOGISTIC:
      case POISSON: return eval_glm(th, grad, propto);
      case HIER_NORMAL: return eval_hier_normal(th, grad, propto, jacobian);
      case HIER_LOGISTIC: return eval_hier_logistic(th, grad, propto, jacobian);
    }
    return std::numeric_limits<double>::quiet_NaN();
  }

  // normal(0, s) prior on n consecutive coordinates.
  static void normal_prior(const double* th, double* grad, int n, double s,
                           bool propto, CSum& lp) {
    for (int i = 0; i < n; ++i) {
      double z = th[i] / s;
      lp.add(-0.5 * z * z);
      if (!propto) lp.add(-std::log(s) - LOG_SQRT_2PI);
      if (grad) grad[i] += -th[i] / (s * s);
    }
  }

  // Logistic (bernoulli_logit) or Poisson (poisson_log) GLM:
  //   eta_n = alpha + x_n . beta
  //   logistic: y eta - log1p_exp(eta);  d/deta = y - inv_logit(eta)
  //   poisson : y eta - exp(eta) [- lgamma(y+1)];  d/deta = y - exp(eta)
  // prior: every coordinate ~ normal(0, hp[0]).
  // compensated != 0: Neumaier sums over rows (the parity reference);
  // compensated == 0: plain sums, vectorisable (the timed CPU baseline).
  double eval_glm(const double* th, double* grad, bool propto) const {
    return compensated ? eval_glm_t<true>(th, grad, propto)
                       : eval_glm_t<false>(th, grad, propto);
  }

  template <bool COMP>
  double eval_glm_t(const double* th, double* grad, bool propto) const {
    const int off = intercept ? 1 : 0;
    const double alpha = intercept ? th[0] : 0.0;
    const double* beta = th + off;
    CSum lp;
    double lp_plain = 0.0;
    std::vector<CSum> g(grad && COMP ? D : 0);
    Vec gp(grad && !COMP ? D : 0, 0.0);
    for (int n = 0; n < N; ++n) {
      const double* xn = &X[(size_t)n * K];
      double eta;
      if (COMP) {
        eta = alpha;
        for (int k = 0; k < K; ++k) eta += xn[k] * beta[k];
      } else {
        double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        int k = 0;
        for (; k + 4 <= K; k += 4) {
          a0 += xn[k] * beta[k];
          a1 += xn[k + 1] * beta[k + 1];
          a2 += xn[k + 2] * beta[k + 2];
          a3 += xn[k + 3] * beta[k + 3];
        }
        for (; k < K; ++k) a0 += xn[k] * beta[k];
        eta = alpha + ((a0 + a1) + (a2 + a3));
      }
      double term, r;
      if (kind == LOGISTIC) {
        double e = std::exp(-std::fabs(eta));
        term = y[n] * eta - ((eta > 0 ? eta : 0.0) + std::log1p(e));
        r = y[n] - (eta >= 0 ? 1.0 / (1.0 + e) : e / (1.0 + e));
      } else {
        double mu = std::exp(eta);
        term = y[n] * eta - mu;
        if (!propto) term -= std::lgamma(y[n] + 1.0);
        r = y[n] - mu;
      }
      if (COMP) lp.add(term); else lp_plain += term;
      if (grad) {
        if (COMP) {
          if (intercept) g[0].add(r);
          for (int k = 0; k < K; ++k) g[off + k].add(xn[k] * r);
        } else {
          if (intercept) gp[0] += r;
          double* gk = gp.data() + off;
          for (int k = 0; k < K; ++k) gk[k] += xn[k] * r;
        }
      }
    }
    if (!COMP) lp.add(lp_plain);
    if (grad)
      for (int d = 0; d < D; ++d) grad[d] = COMP ? g[d].value() : gp[d];
    normal_prior(th, grad, D, hpv(0, kind == LOGISTIC ? 2.5 : 1.0), propto, lp);
    return lp.value();
  }

  // Non-centered hierarchical normal, theta = (mu, log tau, log sigma, z[J], beta[K]):
  //   eta_n = mu + tau z_{g(n)} + x_n . beta,  y_n ~ normal(eta_n, sigma)
  //   mu ~ normal(0, hp0), tau ~ normal(0, hp1) (tau>0), sigma ~ normal(0, hp2)
  //   (sigma>0), z ~ normal(0,1), beta ~ normal(0, hp3).
  double eval_hier_normal(const double* th, double* grad, bool propto,
                          bool jacobian) const {
    const double mu = th[0], ut = th[1], us = th[2];
    const double tau = std::exp(ut), sigma = std::exp(us);
    const double* z = th + 3;
    const double* beta = th + 3 + J;
    const double s_mu = hpv(0, 5.0), s_tau = hpv(1, 1.0), s_sig = hpv(2, 1.0),
                 s_beta = hpv(3, 1.0);
    const double inv_s2 = 1.0 / (sigma * sigma);
    CSum lp, gmu, gtau, gsq;
    std::vector<CSum> gz(grad ? J : 0), gb(grad ? K : 0);
    for (int n = 0; n < N; ++n) {
      const double* xn = &X[(size_t)n * K];
      int j = group[n];
      double eta = mu + tau * z[j];
      for (int k = 0; k < K; ++k) eta += xn[k] * beta[k];
      double e = y[n] - eta;
      lp.add(-0.5 * e * e * inv_s2);
      if (grad) {
        double r = e * inv_s2;
        gmu.add(r);
        gz[j].add(r);
        gtau.add(r * z[j]);
        gsq.add(e * e);
        for (int k = 0; k < K; ++k) gb[k].add(xn[k] * r);
      }
    }
    lp.add(-(double)N * us);  // -N log sigma
    if (!propto) lp.add(-(double)N * LOG_SQRT_2PI);
    // priors
    lp.add(-0.5 * (mu / s_mu) * (mu / s_mu));
    lp.add(-0.5 * (tau / s_tau) * (tau / s_tau));
    lp.add(-0.5 * (sigma / s_sig) * (sigma / s_sig));
    if (!propto)
      lp.add(-std::log(s_mu) - std::log(s_tau) - std::log(s_sig) - 3 * LOG_SQRT_2PI);
    for (int j = 0; j < J; ++j) {
      lp.add(-0.5 * z[j] * z[j]);
      if (!propto) lp.add(-LOG_SQRT_2PI);
    }
    for (int k = 0; k < K; ++k) {
      double b = beta[k] / s_beta;
      lp.add(-0.5 * b * b);
      if (!propto) lp.add(-std::log(s_beta) - LOG_SQRT_2PI);
    }
    if (jacobian) {
      lp.add(ut);
      lp.add(us);
    }
    if (grad) {
      grad[0] = gmu.value() - mu / (s_mu * s_mu);
      double dtau = gtau.value() - tau / (s_tau * s_tau);
      grad[1] = tau * dtau + (jacobian ? 1.0 : 0.0);
      double dsig = -(double)N / sigma + gsq.value() / (sigma * sigma * sigma) -
                    sigma / (s_sig * s_sig);
      grad[2] = sigma * dsig + (jacobian ? 1.0 : 0.0);
      for (int j = 0; j < J; ++j) grad[3 + j] = tau * gz[j].value() - z[j];
      for (int k = 0; k < K; ++k)
        grad[3 + J + k] = gb[k].value() - beta[k] / (s_beta * s_beta);
    }
    return lp.value();
  }

  // Non-centered hierarchical logistic, theta = (alpha, log tau, z[J], beta[K]):
  //   eta_n = alpha + tau z_{g(n)} + x_n . beta,  y_n ~ bernoulli_logit(eta_n)
  //   alpha ~ normal(0, hp0), tau ~ normal(0, hp1) (tau>0), z ~ normal(0,1),
  //   beta ~ normal(0, hp2).
  double eval_hier_logistic(const double* th, double* grad, bool propto,
                            bool jacobian) const {
    const double alpha = th[0], ut = th[1];
    const double tau = std::exp(ut);
    const double* z = th + 2;
    const double* beta = th + 2 + J;
    const double s_a = hpv(0, 2.5), s_tau = hpv(1, 1.0), s_beta = hpv(2, 2.5);
    CSum lp, ga, gtau;
    std::vector<CSum> gz(grad ? J : 0), gb(grad ? K : 0);
    for (int n = 0; n < N; ++n) {
      const double* xn = &X[(size_t)n * K];
      int j = group[n];
      double eta = alpha + tau * z[j];
      for (int k = 0; k < K; ++k) eta += xn[k] * beta[k];
      lp.add(y[n] * eta - log1p_exp(eta));
      if (grad) {
        double r = y[n] - inv_logit(eta);
        ga.add(r);
        gz[j].add(r);
        gtau.add(r * z[j]);
        for (int k = 0; k < K; ++k) gb[k].add(xn[k] * r);
      }
    }
    lp.add(-0.5 * (alpha / s_a) * (alpha / s_a));
    lp.add(-0.5 * (tau / s_tau) * (tau / s_tau));
    if (!propto) lp.add(-std::log(s_a) - std::log(s_tau) - 2 * LOG_SQRT_2PI);
    for (int j = 0; j < J; ++j) {
      lp.add(-0.5 * z[j] * z[j]);
      if (!propto) lp.add(-LOG_SQRT_2PI);
    }
    for (int k = 0; k < K; ++k) {
      double b = beta[k] / s_beta;
      lp.add(-0.5 * b * b);
      if (!propto) lp.add(-std::log(s_beta) - LOG_SQRT_2PI);
    }
    if (jacobian) lp.add(ut);
    if (grad) {
      grad[0] = ga.value() - alpha / (s_a * s_a);
      grad[1] = tau * (gtau.value() - tau / (s_tau * s_tau)) + (jacobian ? 1.0 : 0.0);
      for (int j = 0; j < J; ++j) grad[2 + j] = tau * gz[j].value() - z[j];
      for (int k = 0; k < K; ++k)
        grad[2 + J + k] = gb[k].value() - beta[k] / (s_beta * s_beta);
    }
    return lp.value();
  }

  // write_array: unconstrained -> constrained (tau, sigma = exp).
  void write_array(const double* th, double* out) const {
    for (int d = 0; d < D; ++d) out[d] = th[d];
    if (kind == HIER_NORMAL) {
      out[1] = std::exp(th[1]);
      out[2] = std::exp(th[2]);
    } else if (kind == HIER_LOGISTIC) {
      out[1] = std::exp(th[1]);
    }
  }
};

// ---------------------------------------------------------------- draws
class DrawSource {
 public:
  virtual ~DrawSource() {}
  virtual double uniform() = 0;
  virtual double normal() = 0;
  uint64_t n_uniform = 0, n_normal = 0;
};

class PhiloxSource : public DrawSource {
 public:
  PhiloxSource(uint32_t seed, uint32_t chain) : seed_(seed), chain_(chain) {}
  double uniform() override { return gbds_uniform_at(seed_, chain_, n_uniform++); }
  double normal() override { return gbds_normal_at(seed_, chain_, n_normal++); }

 private:
  uint32_t seed_, chain_;
};

class ScriptedSource : public DrawSource {
 public:
  ScriptedSource(const double* u, int nu, const double* z, int nz)
      : u_(u, u + nu), z_(z, z + nz) {}
  double uniform() override {
    if (n_uniform >= u_.size()) throw std::runtime_error("scripted uniforms exhausted");
    return u_[n_uniform++];
  }
  double normal() override {
    if (n_normal >= z_.size()) throw std::runtime_error("scripted normals exhausted");
    return z_[n_normal++];
  }

 private:
  Vec u_, z_;
};

// ---------------------------------------------------------------- logger
struct Logger {
  std::vector<std::string> lines;  // "level|message"
  void info(const std::string& s) { lines.push_back("info|" + s); }
  void warn(const std::string& s) { lines.push_back("warn|" + s); }
  void error(const std::string& s) { lines.push_back("error|" + s); }
};

// ---------------------------------------------------------------- hamiltonians
struct PsPoint {
  Vec q, p, g;
  double V = 0.0;
  explicit PsPoint(int n = 0) : q(n, 0.0), p(n, 0.0), g(n, 0.0) {}
};

class Hamiltonian {
 public:
  virtual ~Hamiltonian() {}
  virtual double T(PsPoint& z) = 0;
  double V(PsPoint& z) { return z.V; }
  double H(PsPoint& z) { return T(z) + V(z); }
  virtual Vec dtau_dp(PsPoint& z) = 0;
  virtual Vec dphi_dq(PsPoint& z) = 0;
  virtual void sample_p(PsPoint& z, DrawSource& rng) = 0;
  virtual void init(PsPoint& z) { update_potential_gradient(z); }
  virtual void update_potential_gradient(PsPoint& z) = 0;
};

// diag_e_metric (diag_e_metric.hpp:20-50) over base_hamiltonian
// (base_hamiltonian.hpp:61-70): V = -log p, g = -grad log p.
class DiagEHamiltonian : public Hamiltonian {
 public:
  DiagEHamiltonian(const Model& m, int D) : model_(m), inv_metric(D, 1.0) {}
  double T(PsPoint& z) override {
    Vec t(z.p.size());
    for (size_t i = 0; i < t.size(); ++i) t[i] = inv_metric[i] * z.p[i];
    return 0.5 * dot(z.p, t);
  }
  Vec dtau_dp(PsPoint& z) override {
    Vec t(z.p.size());
    for (size_t i = 0; i < t.size(); ++i) t[i] = inv_metric[i] * z.p[i];
    return t;
  }
  Vec dphi_dq(PsPoint& z) override { return z.g; }
  void sample_p(PsPoint& z, DrawSource& rng) override {
    for (size_t i = 0; i < z.p.size(); ++i)
      z.p[i] = rng.normal() / std::sqrt(inv_metric[i]);
  }
  void update_potential_gradient(PsPoint& z) override {
    Vec grad(z.q.size());
    double lp = model_.eval(z.q.data(), grad.data(), true, true);
    ++n_grad;
    z.V = std::isfinite(lp) ? -lp : (std::isnan(lp) ? lp : INF);
    for (size_t i = 0; i < grad.size(); ++i) z.g[i] = -grad[i];
  }
  const Model& model_;
  Vec inv_metric;
  long long n_grad = 0;
};

// Cholesky factor of the lower triangle of a (row-major n x n): l lower
// with a = l l^T, column by column, every element's dot product summed in
// ascending k (the device computes the same sums in the same order).
// Returns false when a pivot is not positive (not positive definite).
static bool cholesky_lower(const Vec& a, int n, Vec& l) {
  l.assign((size_t)n * n, 0.0);
  bool ok = true;
  for (int j = 0; j < n; ++j) {
    Vec s(n, 0.0);
    for (int i = j; i < n; ++i) {
      double v = a[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) v = v - l[(size_t)i * n + k] * l[(size_t)j * n + k];
      s[i] = v;
    }
    if (!(s[j] > 0)) ok = false;
    const double d = std::sqrt(s[j]);
    l[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; ++i) l[(size_t)i * n + j] = s[i] / d;
  }
  return ok;
}

// dense_e_metric (dense_e_metric.hpp:17-62): T = 1/2 p . (A p), dtau_dp = A p
// (row i summed over ascending j), sample_p: p = U^{-1} u with A = U^T U,
// U = L^T (the reference's inv_e_metric_.llt().matrixU().solve(u)), solved
// column by column from the last: p_j = r_j / U_jj, then r_i -= U_ij p_j.
class DenseEHamiltonian : public Hamiltonian {
 public:
  DenseEHamiltonian(const Model& m, int D) : model_(m), D_(D) {
    Vec eye((size_t)D * D, 0.0);
    for (int i = 0; i < D; ++i) eye[(size_t)i * D + i] = 1.0;
    set_metric(eye);
  }
  bool set_metric(const Vec& a) {
    inv_metric = a;
    return cholesky_lower(inv_metric, D_, chol);
  }
  Vec mul(const Vec& p) const {
    Vec t(D_);
    for (int i = 0; i < D_; ++i) {
      double v = 0.0;
      for (int j = 0; j < D_; ++j) v = v + inv_metric[(size_t)i * D_ + j] * p[j];
      t[i] = v;
    }
    return t;
  }
  double T(PsPoint& z) override { return 0.5 * dot(z.p, mul(z.p)); }
  Vec dtau_dp(PsPoint& z) override { return mul(z.p); }
  Vec dphi_dq(PsPoint& z) override { return z.g; }
  void sample_p(PsPoint& z, DrawSource& rng) override {
    Vec r(D_);
    for (int i = 0; i < D_; ++i) r[i] = rng.normal();
    for (int j = D_ - 1; j >= 0; --j) {
      const double pj = r[j] / chol[(size_t)j * D_ + j];
      z.p[j] = pj;
      for (int i = 0; i < j; ++i) r[i] = r[i] - chol[(size_t)j * D_ + i] * pj;
    }
  }
  void update_potential_gradient(PsPoint& z) override {
    Vec grad(z.q.size());
    double lp = model_.eval(z.q.data(), grad.data(), true, true);
    ++n_grad;
    z.V = std::isfinite(lp) ? -lp : (std::isnan(lp) ? lp : INF);
    for (size_t i = 0; i < grad.size(); ++i) z.g[i] = -grad[i];
  }
  const Model& model_;
  int D_;
  Vec inv_metric;  // row-major D x D
  Vec chol;        // L, row-major, lower
  long long n_grad = 0;
};

// mock_hamiltonian (src/test/unit/mcmc/hmc/mock_hmc.hpp:38-63)
class MockHamiltonian : public Hamiltonian {
 public:
  double T(PsPoint&) override { return 0; }
  Vec dtau_dp(PsPoint& z) override { return z.q; }
  Vec dphi_dq(PsPoint& z) override { return Vec(z.q.size(), 0.0); }
  void sample_p(PsPoint&, DrawSource&) override {}
  void update_potential_gradient(PsPoint& z) override {
    z.V = -0.0;  // mock_model::log_prob == 0
    for (auto& v : z.g) v = -0.0;
  }
};

// divergent_hamiltonian (src/test/unit/mcmc/hmc/nuts/base_nuts_test.cpp:58-91)
class DivergentHamiltonian : public Hamiltonian {
 public:
  double T(PsPoint&) override { return 0; }
  Vec dtau_dp(PsPoint& z) override { return Vec(z.q.size(), 0.0); }
  Vec dphi_dq(PsPoint& z) override { return Vec(z.q.size(), 0.0); }
  void sample_p(PsPoint&, DrawSource&) override {}
  void init(PsPoint& z) override { z.V = 0; }
  void update_potential_gradient(PsPoint& z) override { z.V += 500; }
};

// ---------------------------------------------------------------- integrators
class Integrator {
 public:
  virtual ~Integrator() {}
  virtual void evolve(PsPoint& z, Hamiltonian& h, double eps) = 0;
};

// expl_leapfrog (expl_leapfrog.hpp:16-32) driven by base_leapfrog::evolve
// (base_leapfrog.hpp:17-22).
class ExplLeapfrog : public Integrator {
 public:
  void evolve(PsPoint& z, Hamiltonian& h, double eps) override {
    update_p(z, h, 0.5 * eps);
    Vec t = h.dtau_dp(z);
    for (size_t i = 0; i < z.q.size(); ++i) z.q[i] = z.q[i] + eps * t[i];
    h.update_potential_gradient(z);
    update_p(z, h, 0.5 * eps);
  }

 private:
  static void update_p(PsPoint& z, Hamiltonian& h, double e) {
    Vec g = h.dphi_dq(z);
    for (size_t i = 0; i < z.p.size(); ++i) z.p[i] = z.p[i] - e * g[i];
  }
};

// mock_integrator (mock_hmc.hpp:66-75)
class MockIntegrator : public Integrator {
 public:
  void evolve(PsPoint& z, Hamiltonian&, double eps) override {
    for (size_t i = 0; i < z.q.size(); ++i) z.q[i] += eps * z.p[i];
  }
};

// ---------------------------------------------------------------- sampler
struct Sample {
  Vec q;
  double log_prob = 0, accept_stat = 0;
};

// base_hmc + base_nuts (base_hmc.hpp:28-215, base_nuts.hpp:19-361)
class Nuts {
 public:
  Nuts(Hamiltonian& h, Integrator& in, DrawSource& r, int D)
      : ham(h), integ(in), rng(r), z(D) {}
  virtual ~Nuts() {}

  Hamiltonian& ham;
  Integrator& integ;
  DrawSource& rng;
  PsPoint z;
  double nom_epsilon = 0.1, epsilon = 0.1, epsilon_jitter = 0.0;
  int depth = 0, max_depth = 5;
  double max_deltaH = 1000;
  int n_leapfrog = 0;
  bool divergent = false;
  double energy = 0;

  void set_nominal_stepsize(double e) {
    if (e > 0) nom_epsilon = e;
  }
  void set_stepsize_jitter(double j) {
    if (j > 0 && j < 1) epsilon_jitter = j;
  }
  void set_max_depth(int d) {
    if (d > 0) max_depth = d;
  }

  // base_hmc::sample_stepsize (base_hmc.hpp:195-200)
  void sample_stepsize() {
    epsilon = nom_epsilon;
    if (epsilon_jitter)
      epsilon *= 1.0 + epsilon_jitter * (2.0 * rng.uniform() - 1.0);
  }

  virtual bool compute_criterion(Vec& p_sharp_minus, Vec& p_sharp_plus, Vec& rho) {
    return dot(p_sharp_plus, rho) > 0 && dot(p_sharp_minus, rho) > 0;
  }

  // base_hmc::init_stepsize (base_hmc.hpp:93-161)
  void init_stepsize() {
    PsPoint z_init(z);
    if (z.q.empty()) {
      nom_epsilon = std::numeric_limits<double>::quiet_NaN();
      return;
    }
    if (nom_epsilon == 0 || nom_epsilon > 1e7 || std::isnan(nom_epsilon)) return;
    ham.sample_p(z, rng);
    ham.init(z);
    double H0 = ham.H(z);
    integ.evolve(z, ham, nom_epsilon);
    ++n_stepsize_trials;
    double h = ham.H(z);
    if (std::isnan(h)) h = INF;
    double delta_H = H0 - h;
    int direction = delta_H > std::log(0.8) ? 1 : -1;
    while (1) {
      z = z_init;
      ham.sample_p(z, rng);
      ham.init(z);
      double H0b = ham.H(z);
      integ.evolve(z, ham, nom_epsilon);
      ++n_stepsize_trials;
      double hb = ham.H(z);
      if (std::isnan(hb)) hb = INF;
      double dH = H0b - hb;
      if ((direction == 1) && !(dH > std::log(0.8)))
        break;
      else if ((direction == -1) && !(dH < std::log(0.8)))
        break;
      else
        nom_epsilon = direction == 1 ? 2.0 * nom_epsilon : 0.5 * nom_epsilon;
      if (nom_epsilon > 1e7)
        throw std::runtime_error("Posterior is improper. Please check your model.");
      if (nom_epsilon == 0)
        throw std::runtime_error(
            "No acceptably small step size could be found. Perhaps the "
            "posterior is not continuous?");
    }
    z = z_init;
  }

  // base_nuts::transition (base_nuts.hpp:78-204)
  Sample transition(const Sample& init_sample) {
    sample_stepsize();
    z.q = init_sample.q;
    ham.sample_p(z, rng);
    ham.init(z);

    PsPoint z_fwd(z), z_bck(z), z_sample(z), z_propose(z);
    Vec p_fwd_fwd = z.p;
    Vec p_sharp_fwd_fwd = ham.dtau_dp(z);
    Vec p_fwd_bck = z.p;
    Vec p_sharp_fwd_bck = p_sharp_fwd_fwd;
    Vec p_bck_fwd = z.p;
    Vec p_sharp_bck_fwd = p_sharp_fwd_fwd;
    Vec p_bck_bck = z.p;
    Vec p_sharp_bck_bck = p_sharp_fwd_fwd;
    Vec rho = z.p;
    double log_sum_weight = 0;
    double H0 = ham.H(z);
    int n_lf = 0;
    double sum_metro_prob = 0;
    depth = 0;
    divergent = false;
    const size_t D = rho.size();

    while (depth < max_depth) {
      Vec rho_fwd(D, 0.0), rho_bck(D, 0.0);
      bool valid_subtree = false;
      double log_sum_weight_subtree = -INF;
      if (rng.uniform() > 0.5) {
        z = z_fwd;
        rho_bck = rho;
        p_bck_fwd = p_fwd_fwd;
        p_sharp_bck_fwd = p_sharp_fwd_fwd;
        valid_subtree = build_tree(depth, z_propose, p_sharp_fwd_bck, p_sharp_fwd_fwd,
                                   rho_fwd, p_fwd_bck, p_fwd_fwd, H0, 1, n_lf,
                                   log_sum_weight_subtree, sum_metro_prob);
        z_fwd = z;
      } else {
        z = z_bck;
        rho_fwd = rho;
        p_fwd_bck = p_bck_bck;
        p_sharp_fwd_bck = p_sharp_bck_bck;
        valid_subtree = build_tree(depth, z_propose, p_sharp_bck_fwd, p_sharp_bck_bck,
                                   rho_bck, p_bck_fwd, p_bck_bck, H0, -1, n_lf,
                                   log_sum_weight_subtree, sum_metro_prob);
        z_bck = z;
      }
      if (!valid_subtree) break;
      ++depth;
      if (log_sum_weight_subtree > log_sum_weight) {
        z_sample = z_propose;
      } else {
        double accept_prob = std::exp(log_sum_weight_subtree - log_sum_weight);
        if (rng.uniform() < accept_prob) z_sample = z_propose;
      }
      log_sum_weight = log_sum_exp(log_sum_weight, log_sum_weight_subtree);
      for (size_t i = 0; i < D; ++i) rho[i] = rho_bck[i] + rho_fwd[i];
      bool persist = compute_criterion(p_sharp_bck_bck, p_sharp_fwd_fwd, rho);
      Vec rho_ext(D);
      for (size_t i = 0; i < D; ++i) rho_ext[i] = rho_bck[i] + p_fwd_bck[i];
      persist &= compute_criterion(p_sharp_bck_bck, p_sharp_fwd_bck, rho_ext);
      for (size_t i = 0; i < D; ++i) rho_ext[i] = rho_fwd[i] + p_bck_fwd[i];
      persist &= compute_criterion(p_sharp_bck_fwd, p_sharp_fwd_fwd, rho_ext);
      if (!persist) break;
    }
    n_leapfrog = n_lf;
    total_leapfrogs += n_lf;
    double accept_prob = sum_metro_prob / static_cast<double>(n_lf);
    z = z_sample;
    energy = ham.H(z);
    Sample s;
    s.q = z.q;
    s.log_prob = -z.V;
    s.accept_stat = accept_prob;
    return s;
  }

  // base_nuts::build_tree (base_nuts.hpp:247-352)
  bool build_tree(int d, PsPoint& z_propose, Vec& p_sharp_beg, Vec& p_sharp_end,
                  Vec& rho, Vec& p_beg, Vec& p_end, double H0, double sign,
                  int& n_lf, double& log_sum_weight, double& sum_metro_prob) {
    const size_t D = rho.size();
    if (d == 0) {
      integ.evolve(z, ham, sign * epsilon);
      ++n_lf;
      double h = ham.H(z);
      if (std::isnan(h)) h = INF;
      if ((h - H0) > max_deltaH) divergent = true;
      log_sum_weight = log_sum_exp(log_sum_weight, H0 - h);
      if (H0 - h > 0)
        sum_metro_prob += 1;
      else
        sum_metro_prob += std::exp(H0 - h);
      z_propose = z;
      p_sharp_beg = ham.dtau_dp(z);
      p_sharp_end = p_sharp_beg;
      for (size_t i = 0; i < D; ++i) rho[i] += z.p[i];
      p_beg = z.p;
      p_end = p_beg;
      return !divergent;
    }
    double log_sum_weight_init = -INF;
    Vec p_init_end(D), p_sharp_init_end(D), rho_init(D, 0.0);
    bool valid_init = build_tree(d - 1, z_propose, p_sharp_beg, p_sharp_init_end,
                                 rho_init, p_beg, p_init_end, H0, sign, n_lf,
                                 log_sum_weight_init, sum_metro_prob);
    if (!valid_init) return false;
    PsPoint z_propose_final(z);
    double log_sum_weight_final = -INF;
    Vec p_final_beg(D), p_sharp_final_beg(D), rho_final(D, 0.0);
    bool valid_final = build_tree(d - 1, z_propose_final, p_sharp_final_beg,
                                  p_sharp_end, rho_final, p_final_beg, p_end, H0,
                                  sign, n_lf, log_sum_weight_final, sum_metro_prob);
    if (!valid_final) return false;
    double log_sum_weight_subtree = log_sum_exp(log_sum_weight_init, log_sum_weight_final);
    log_sum_weight = log_sum_exp(log_sum_weight, log_sum_weight_subtree);
    if (log_sum_weight_final > log_sum_weight_subtree) {
      z_propose = z_propose_final;
    } else {
      double accept_prob = std::exp(log_sum_weight_final - log_sum_weight_subtree);
      if (rng.uniform() < accept_prob) z_propose = z_propose_final;
    }
    Vec rho_subtree(D);
    for (size_t i = 0; i < D; ++i) rho_subtree[i] = rho_init[i] + rho_final[i];
    for (size_t i = 0; i < D; ++i) rho[i] += rho_subtree[i];
    bool persist = compute_criterion(p_sharp_beg, p_sharp_end, rho_subtree);
    for (size_t i = 0; i < D; ++i) rho_subtree[i] = rho_init[i] + p_final_beg[i];
    persist &= compute_criterion(p_sharp_beg, p_sharp_final_beg, rho_subtree);
    for (size_t i = 0; i < D; ++i) rho_subtree[i] = rho_final[i] + p_init_end[i];
    persist &= compute_criterion(p_sharp_init_end, p_sharp_end, rho_subtree);
    return persist;
  }

  long long n_stepsize_trials = 0;
  long long total_leapfrogs = 0;
};

// ---------------------------------------------------------------- adaptation
// stepsize_adaptation (stepsize_adaptation.hpp:13-73)
struct StepsizeAdaptation {
  double counter = 0, s_bar = 0, x_bar = 0;
  double mu = 0.5, delta = 0.5, gamma = 0.05, kappa = 0.75, t0 = 10;
  void restart() { counter = 0; s_bar = 0; x_bar = 0; }
  void set_mu(double m) { mu = m; }
  void set_delta(double d) { if (d > 0 && d < 1) delta = d; }
  void set_gamma(double g) { if (g > 0) gamma = g; }
  void set_kappa(double k) { if (k > 0) kappa = k; }
  void set_t0(double t) { if (t > 0) t0 = t; }
  void learn_stepsize(double& epsilon, double adapt_stat) {
    ++counter;
    adapt_stat = adapt_stat > 1 ? 1 : adapt_stat;
    const double eta = 1.0 / (counter + t0);
    s_bar = (1.0 - eta) * s_bar + eta * (delta - adapt_stat);
    const double x = mu - s_bar * std::sqrt(counter) / gamma;
    const double x_eta = std::pow(counter, -kappa);
    x_bar = (1.0 - x_eta) * x_bar + x_eta * x;
    epsilon = std::exp(x);
  }
  void complete_adaptation(double& epsilon) { epsilon = std::exp(x_bar); }
};

// windowed_adaptation (windowed_adaptation.hpp:14-110); unsigned arithmetic
// as in the reference (adapt_next_window_ wraps when the schedule is unset).
struct WindowedAdaptation {
  std::string name = "variance";
  unsigned num_warmup = 0, adapt_init_buffer = 0, adapt_term_buffer = 0,
           adapt_base_window = 0;
  unsigned adapt_window_counter = 0, adapt_next_window = 0, adapt_window_size = 0;
  WindowedAdaptation() { restart(); }
  void restart() {
    adapt_window_counter = 0;
    adapt_window_size = adapt_base_window;
    adapt_next_window = adapt_init_buffer + adapt_window_size - 1;
  }
  void set_window_params(unsigned nw, unsigned ib, unsigned tb, unsigned bw,
                         Logger& logger) {
    if (nw < 20) {
      logger.info("WARNING: No " + name + " estimation is");
      logger.info("         performed for num_warmup < 20");
      logger.info("");
      return;
    }
    if (ib + bw + tb > nw) {
      logger.info("WARNING: There aren't enough warmup iterations to fit the");
      logger.info(std::string("         three stages of adaptation as currently") +
                  " configured.");
      num_warmup = nw;
      adapt_init_buffer = 0.15 * nw;
      adapt_term_buffer = 0.1 * nw;
      adapt_base_window = nw - (adapt_init_buffer + adapt_term_buffer);
      logger.info("         Reducing each adaptation stage to 15%/75%/10% of");
      logger.info("         the given number of warmup iterations:");
      std::ostringstream a, b, c;
      a << "           init_buffer = " << adapt_init_buffer;
      b << "           adapt_window = " << adapt_base_window;
      c << "           term_buffer = " << adapt_term_buffer;
      logger.info(a.str());
      logger.info(b.str());
      logger.info(c.str());
      logger.info("");
      return;
    }
    num_warmup = nw;
    adapt_init_buffer = ib;
    adapt_term_buffer = tb;
    adapt_base_window = bw;
    restart();
  }
  bool adaptation_window() const {
    return (adapt_window_counter >= adapt_init_buffer) &&
           (adapt_window_counter < num_warmup - adapt_term_buffer) &&
           (adapt_window_counter != num_warmup);
  }
  bool end_adaptation_window() const {
    return (adapt_window_counter == adapt_next_window) &&
           (adapt_window_counter != num_warmup);
  }
  void compute_next_window() {
    if (adapt_next_window == num_warmup - adapt_term_buffer - 1) return;
    adapt_window_size *= 2;
    adapt_next_window = adapt_window_counter + adapt_window_size;
    if (adapt_next_window == num_warmup - adapt_term_buffer - 1) return;
    unsigned next_window_boundary = adapt_next_window + 2 * adapt_window_size;
    if (next_window_boundary >= num_warmup - adapt_term_buffer)
      adapt_next_window = num_warmup - adapt_term_buffer - 1;
  }
};

// welford_var_estimator (Stan Math; used at var_adaptation.hpp:49)
struct Welford {
  double n = 0;
  Vec m, m2;
  explicit Welford(int d = 0) : m(d, 0.0), m2(d, 0.0) {}
  void restart() {
    n = 0;
    std::fill(m.begin(), m.end(), 0.0);
    std::fill(m2.begin(), m2.end(), 0.0);
  }
  void add_sample(const Vec& q) {
    n += 1;
    for (size_t i = 0; i < q.size(); ++i) {
      double delta = q[i] - m[i];
      m[i] += delta / n;
      m2[i] += (q[i] - m[i]) * delta;
    }
  }
  void sample_variance(Vec& var) const {
    if (n > 1)
      for (size_t i = 0; i < var.size(); ++i) var[i] = m2[i] / (n - 1.0);
  }
};

// var_adaptation (var_adaptation.hpp:17-46)
struct VarAdaptation : WindowedAdaptation {
  Welford est;
  explicit VarAdaptation(int d) : est(d) {}
  bool learn_variance(Vec& var, const Vec& q) {
    if (adaptation_window()) est.add_sample(q);
    if (end_adaptation_window()) {
      compute_next_window();
      est.sample_variance(var);
      double n = est.n;
      for (auto& v : var) v = (n / (n + 5.0)) * v + 1e-3 * (5.0 / (n + 5.0));
      for (auto v : var)
        if (!std::isfinite(v))
          throw std::runtime_error(
              "Numerical overflow in metric adaptation. This occurs when the "
              "sampler encounters extreme values on the unconstrained space; "
              "this may happen when the posterior density function is too wide "
              "or improper. There may be problems with your model specification.");
      est.restart();
      ++adapt_window_counter;
      return true;
    }
    ++adapt_window_counter;
    return false;
  }
};

// adapt_diag_e_nuts (adapt_diag_e_nuts.hpp:25-48) on top of diag_e_nuts
class AdaptDiagENuts : public Nuts {
 public:
  AdaptDiagENuts(DiagEHamiltonian& h, Integrator& in, DrawSource& r, int D)
      : Nuts(h, in, r, D), dham(h), var_adapt(D) {}
  DiagEHamiltonian& dham;
  StepsizeAdaptation ss_adapt;
  VarAdaptation var_adapt;
  bool adapt_flag = false;
  Sample adapt_transition(const Sample& init) {
    Sample s = transition(init);
    if (adapt_flag) {
      ss_adapt.learn_stepsize(nom_epsilon, s.accept_stat);
      bool update = var_adapt.learn_variance(dham.inv_metric, z.q);
      if (update) {
        init_stepsize();
        ss_adapt.set_mu(std::log(10 * nom_epsilon));
        ss_adapt.restart();
      }
    }
    return s;
  }
  void disengage_adaptation() {
    adapt_flag = false;
    ss_adapt.complete_adaptation(nom_epsilon);
  }
};

// welford_covar_estimator (Stan Math; used at covar_adaptation.hpp:51):
// m += delta / n, m2 += (q - m) delta^T, covariance m2 / (n - 1) when n > 1.
struct WelfordCovar {
  double n = 0;
  int d = 0;
  Vec m, m2;
  explicit WelfordCovar(int dim = 0) : d(dim), m(dim, 0.0), m2((size_t)dim * dim, 0.0) {}
  void restart() {
    n = 0;
    std::fill(m.begin(), m.end(), 0.0);
    std::fill(m2.begin(), m2.end(), 0.0);
  }
  void add_sample(const Vec& q) {
    n += 1;
    Vec delta(d);
    for (int i = 0; i < d; ++i) {
      delta[i] = q[i] - m[i];
      m[i] = m[i] + delta[i] / n;
    }
    for (int i = 0; i < d; ++i)
      for (int j = 0; j < d; ++j)
        m2[(size_t)i * d + j] = m2[(size_t)i * d + j] + (q[i] - m[i]) * delta[j];
  }
  void sample_covariance(Vec& covar) const {
    if (n > 1)
      for (size_t k = 0; k < covar.size(); ++k) covar[k] = m2[k] / (n - 1.0);
  }
};

// covar_adaptation (covar_adaptation.hpp:12-57)
struct CovarAdaptation : WindowedAdaptation {
  WelfordCovar est;
  explicit CovarAdaptation(int d) : est(d) {}
  bool learn_covariance(Vec& covar, const Vec& q) {
    if (adaptation_window()) est.add_sample(q);
    if (end_adaptation_window()) {
      compute_next_window();
      est.sample_covariance(covar);
      const double n = est.n;
      const int d = est.d;
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
          double& v = covar[(size_t)i * d + j];
          v = (n / (n + 5.0)) * v + (i == j ? 1e-3 * (5.0 / (n + 5.0)) : 0.0);
        }
      for (double v : covar)
        if (!std::isfinite(v))
          throw std::runtime_error(
              "Numerical overflow in metric adaptation. This occurs when the sampler "
              "encounters extreme values on the unconstrained space; this may happen when "
              "the posterior density function is too wide or improper. There may be "
              "problems with your model specification.");
      est.restart();
      ++adapt_window_counter;
      return true;
    }
    ++adapt_window_counter;
    return false;
  }
};

// adapt_dense_e_nuts (adapt_dense_e_nuts.hpp:25-48) on top of dense_e_nuts
class AdaptDenseENuts : public Nuts {
 public:
  AdaptDenseENuts(DenseEHamiltonian& h, Integrator& in, DrawSource& r, int D)
      : Nuts(h, in, r, D), dham(h), var_adapt(D) {}
  DenseEHamiltonian& dham;
  StepsizeAdaptation ss_adapt;
  CovarAdaptation var_adapt;
  bool adapt_flag = false;
  Sample adapt_transition(const Sample& init) {
    Sample s = transition(init);
    if (adapt_flag) {
      ss_adapt.learn_stepsize(nom_epsilon, s.accept_stat);
      Vec covar = dham.inv_metric;
      bool update = var_adapt.learn_covariance(covar, z.q);
      if (update) {
        dham.set_metric(covar);
        init_stepsize();
        ss_adapt.set_mu(std::log(10 * nom_epsilon));
        ss_adapt.restart();
      }
    }
    return s;
  }
  void disengage_adaptation() {
    adapt_flag = false;
    ss_adapt.complete_adaptation(nom_epsilon);
  }
};

// validate_dense_inv_metric (validate_dense_inv_metric.hpp:20-30) through
// Stan Math's check_pos_definite: finite, symmetric to 1e-8, and a Cholesky
// factorisation with positive pivots.
static bool dense_metric_ok(const Vec& a, int n) {
  for (double v : a)
    if (!std::isfinite(v)) return false;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (std::fabs(a[(size_t)i * n + j] - a[(size_t)j * n + i]) > 1e-8) return false;
  Vec l;
  return n == 0 || cholesky_lower(a, n, l);
}

// ---------------------------------------------------------------- service
struct SamplerConfig {
  int num_warmup = 1000, num_samples = 1000, num_thin = 1, save_warmup = 0,
      refresh = 0;
  double stepsize = 1, stepsize_jitter = 0;
  int max_depth = 10;
  double delta = 0.8, gamma = 0.05, kappa = 0.75, t0 = 10;
  unsigned init_buffer = 75, term_buffer = 50, window = 25;
  double init_radius = 2;
  unsigned seed = 0, init_chain_id = 1;
  int adapt = 1;  // 1: hmc_nuts_diag_e_adapt, 0: hmc_nuts_diag_e
  int dense = 0;  // 1: the dense_e services (hmc_nuts_dense_e_adapt / hmc_nuts_dense_e)
};

// Per-chain output.  Rows: lp__, accept_stat__, stepsize__, treedepth__,
// n_leapfrog__, divergent__, energy__, constrained parameters (D).
struct ChainOut {
  Vec rows;
  Vec unc;           // unconstrained q per saved row
  Vec init;          // unconstrained init used
  double stepsize = 0;
  Vec inv_metric;
  long long n_grad = 0;
  long long n_grad_total = 0;  // every evaluation, incl. the transition-start recompute
  int n_saved = 0;
  int n_warmup_saved = 0;
  int return_code = 0;
  double warm_seconds = 0, sample_seconds = 0;
  uint64_t n_uniform = 0, n_normal = 0;
  Logger log;
};

// util::initialize (initialize.hpp:68-227) with the whole vector either
// supplied (init != nullptr) or drawn uniform(-R, R).
static Vec initialize(const Model& m, const double* init, DrawSource& rng,
                      double init_radius, Logger& logger, long long& n_grad) {
  const int D = m.D;
  bool full = init != nullptr;
  bool zero = init_radius == 0.0;
  int max_tries = (full || zero) ? 1 : 100;
  Vec unc(D), grad(D);
  for (int t = 0; t < max_tries; ++t) {
    if (full) {
      for (int d = 0; d < D; ++d) unc[d] = init[d];
    } else if (zero) {
      for (int d = 0; d < D; ++d) unc[d] = 0.0;
    } else {
      for (int d = 0; d < D; ++d)
        unc[d] = (2.0 * rng.uniform() - 1.0) * init_radius;
    }
    double lp = m.eval(unc.data(), nullptr, false, true);
    if (!std::isfinite(lp)) {
      logger.warn("Rejecting initial value:");
      logger.warn("  Log probability evaluates to log(0), i.e. negative infinity.");
      logger.warn("  Stan can't start sampling from this initial value.");
      continue;
    }
    m.eval(unc.data(), grad.data(), true, true);
    ++n_grad;
    double gs = 0;
    for (double g : grad) gs += g;
    if (!std::isfinite(gs)) {
      logger.warn("Rejecting initial value:");
      logger.warn("  Gradient evaluated at the initial value is not finite.");
      logger.warn("  Stan can't start sampling from this initial value.");
      continue;
    }
    return unc;
  }
  if (!zero) {
    logger.info("");
    std::ostringstream s;
    s << "Initialization between (-" << init_radius << ", " << init_radius
      << ") failed after " << max_tries << " attempts. ";
    logger.error(s.str());
    logger.error(
        " Try specifying initial values, reducing ranges of constrained values, "
        "or reparameterizing the model.");
  }
  throw std::domain_error("Initialization failed.");
}

static void emit_row(const Model& m, const Sample& s, Nuts& sampler, ChainOut& out) {
  out.rows.push_back(s.log_prob);
  out.rows.push_back(s.accept_stat);
  out.rows.push_back(sampler.epsilon);
  out.rows.push_back(sampler.depth);
  out.rows.push_back(sampler.n_leapfrog);
  out.rows.push_back(sampler.divergent ? 1.0 : 0.0);
  out.rows.push_back(sampler.energy);
  Vec c(m.D);
  m.write_array(s.q.data(), c.data());
  out.rows.insert(out.rows.end(), c.begin(), c.end());
  out.unc.insert(out.unc.end(), s.q.begin(), s.q.end());
  out.n_saved++;
}

// One chain of hmc_nuts_diag_e_adapt (hmc_nuts_diag_e_adapt.hpp:57-112) or
// hmc_nuts_diag_e (hmc_nuts_diag_e.hpp:48-100).
// The initial inverse metric: D values (diag_e) or D x D row-major (dense_e),
// ones / identity when none is given; false when it fails the services'
// validation (validate_diag_inv_metric.hpp:18-27, validate_dense_inv_metric.hpp).
static bool set_initial_metric(DiagEHamiltonian& ham, const double* inv_metric, int D) {
  Vec im(D, 1.0);
  if (inv_metric)
    for (int d = 0; d < D; ++d) im[d] = inv_metric[d];
  for (double v : im)
    if (!std::isfinite(v) || !(v > 0)) return false;
  ham.inv_metric = im;
  return true;
}
static bool set_initial_metric(DenseEHamiltonian& ham, const double* inv_metric, int D) {
  if (!inv_metric) return true;
  Vec a(inv_metric, inv_metric + (size_t)D * D);
  if (!dense_metric_ok(a, D)) return false;
  ham.set_metric(a);
  return true;
}

template <class Ham, class Sampler>
static void run_chain_t(const Model& m, const SamplerConfig& cfg, const double* init,
                        const double* inv_metric, unsigned chain_id, ChainOut& out) {
  const int D = m.D;
  PhiloxSource rng(cfg.seed, chain_id);
  Ham ham(m, D);
  ExplLeapfrog integ;
  Sampler sampler(ham, integ, rng, D);
  Vec unc;
  try {
    unc = initialize(m, init, rng, cfg.init_radius, out.log, out.n_grad);
    if (!set_initial_metric(ham, inv_metric, D)) {
      out.log.error("Inverse Euclidean metric not positive definite.");
      throw std::domain_error("Initialization failure");
    }
  } catch (const std::exception& e) {
    out.log.error(e.what());
    out.return_code = 78;
    return;
  }
  out.init = unc;
  sampler.set_nominal_stepsize(cfg.stepsize);
  sampler.set_stepsize_jitter(cfg.stepsize_jitter);
  sampler.set_max_depth(cfg.max_depth);
  if (cfg.adapt) {
    sampler.ss_adapt.set_mu(std::log(10 * cfg.stepsize));
    sampler.ss_adapt.set_delta(cfg.delta);
    sampler.ss_adapt.set_gamma(cfg.gamma);
    sampler.ss_adapt.set_kappa(cfg.kappa);
    sampler.ss_adapt.set_t0(cfg.t0);
    sampler.var_adapt.set_window_params(cfg.num_warmup, cfg.init_buffer,
                                        cfg.term_buffer, cfg.window, out.log);
  }
  try {
    // run_adaptive_sampler.hpp:57-68 / run_sampler.hpp
    if (cfg.adapt) {
      sampler.adapt_flag = true;
      try {
        sampler.z.q = unc;
        sampler.init_stepsize();
      } catch (const std::exception& e) {
        out.log.error("Exception initializing step size.");
        out.log.error(e.what());
        out.n_grad += sampler.n_stepsize_trials;
        return;
      }
    }
    Sample s;
    s.q = unc;
    auto t0 = std::chrono::steady_clock::now();
    for (int mi = 0; mi < cfg.num_warmup; ++mi) {
      s = cfg.adapt ? sampler.adapt_transition(s) : sampler.transition(s);
      if (cfg.save_warmup && (mi % cfg.num_thin) == 0) {
        emit_row(m, s, sampler, out);
        out.n_warmup_saved++;
      }
    }
    auto t1 = std::chrono::steady_clock::now();
    if (cfg.adapt) sampler.disengage_adaptation();
    out.stepsize = sampler.nom_epsilon;
    out.inv_metric = ham.inv_metric;
    for (int mi = 0; mi < cfg.num_samples; ++mi) {
      s = sampler.transition(s);
      if ((mi % cfg.num_thin) == 0) emit_row(m, s, sampler, out);
    }
    auto t2 = std::chrono::steady_clock::now();
    out.warm_seconds = std::chrono::duration<double>(t1 - t0).count();
    out.sample_seconds = std::chrono::duration<double>(t2 - t1).count();
  } catch (const std::exception& e) {
    out.log.error(e.what());
    out.return_code = 70;
  }
  out.n_grad += sampler.n_stepsize_trials + sampler.total_leapfrogs;
  out.n_grad_total = ham.n_grad + out.n_grad - sampler.n_stepsize_trials - sampler.total_leapfrogs;
  out.n_uniform = rng.n_uniform;
  out.n_normal = rng.n_normal;
}

static void run_chain(const Model& m, const SamplerConfig& cfg, const double* init,
                      const double* inv_metric, unsigned chain_id, ChainOut& out) {
  if (cfg.dense)
    run_chain_t<DenseEHamiltonian, AdaptDenseENuts>(m, cfg, init, inv_metric, chain_id, out);
  else
    run_chain_t<DiagEHamiltonian, AdaptDiagENuts>(m, cfg, init, inv_metric, chain_id, out);
}

// ---------------------------------------------------------------- mock tests
// Inspecting samplers from src/test/unit/mcmc/hmc/nuts/base_nuts_test.cpp:12-56.
class MockNuts : public Nuts {
 public:
  using Nuts::Nuts;
  int mode = 0;  // 0 always true, 1 record rho, 2 record edges
  Vec rho_values, minus_values, plus_values;
  bool compute_criterion(Vec& pm, Vec& pp, Vec& rho) override {
    if (mode == 1) rho_values.push_back(rho[0]);
    if (mode == 2) {
      minus_values.push_back(pm[0]);
      plus_values.push_back(pp[0]);
    }
    return true;
  }
};

}  // namespace oracle

// ================================================================ C API
using namespace oracle;

extern "C" {

typedef struct {
  int kind, N, K, J, intercept;
  const double* X;
  const double* y;
  const int* group;
  const double* hp;
  int n_hp;
  int compensated;
} oracle_model_spec;

void* oracle_model_create(const oracle_model_spec* s) {
  try {
    Model* m = new Model();
    m->kind = s->kind;
    m->N = s->N;
    m->K = s->K;
    m->J = s->J;
    m->intercept = s->intercept;
    m->X.assign(s->X, s->X + (size_t)s->N * s->K);
    m->y.assign(s->y, s->y + s->N);
    if (s->group) m->group.assign(s->group, s->group + s->N);
    if (s->hp) m->hp.assign(s->hp, s->hp + s->n_hp);
    m->compensated = s->compensated;
    m->finalize();
    return m;
  } catch (...) {
    return nullptr;
  }
}

void oracle_model_destroy(void* m) { delete static_cast<Model*>(m); }
int oracle_model_dim(void* m) { return static_cast<Model*>(m)->D; }

int oracle_log_prob(void* mp, const double* th, int propto, int jacobian, double* lp) {
  *lp = static_cast<Model*>(mp)->eval(th, nullptr, propto != 0, jacobian != 0);
  return 0;
}

int oracle_log_prob_grad(void* mp, const double* th, int propto, int jacobian,
                         double* lp, double* grad) {
  *lp = static_cast<Model*>(mp)->eval(th, grad, propto != 0, jacobian != 0);
  return 0;
}

int oracle_write_array(void* mp, const double* th, double* out) {
  static_cast<Model*>(mp)->write_array(th, out);
  return 0;
}

// stream 0: uniforms, 1: normals one at a time, 2: the same normals from
// gbds_normal_pair_at (the pairwise form the GPU sampler draws momenta with).
void oracle_draws(unsigned seed, unsigned chain, int stream, unsigned long long start,
                  int n, double* out) {
  for (int i = 0; i < n; ++i) {
    if (stream == 2) {
      double ze, zo;
      gbds_normal_pair_at(seed, chain, (start + i) >> 1, &ze, &zo);
      out[i] = ((start + i) & 1u) ? zo : ze;
    } else {
      out[i] = stream == 0 ? gbds_uniform_at(seed, chain, start + i)
                           : gbds_normal_at(seed, chain, start + i);
    }
  }
}

void oracle_philox(const unsigned* ctr, const unsigned* key, unsigned* out) {
  gbds_block b = gbds_philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = b.w[i];
}

typedef struct {
  int num_warmup, num_samples, num_thin, save_warmup, refresh;
  double stepsize, stepsize_jitter;
  int max_depth;
  double delta, gamma, kappa, t0;
  unsigned init_buffer, term_buffer, window;
  double init_radius;
  unsigned seed, init_chain_id;
  int adapt;
  int dense;  // inverse metrics (in and out) D x D row-major per chain
} oracle_sampler_config;

typedef struct {
  double* rows;        // [n_rows_cap * (7 + D)]
  double* unc;         // [n_rows_cap * D] or NULL
  double* init;        // [D] or NULL
  double* inv_metric;  // [D] or NULL
  double* stepsize;
  long long* n_grad;
  int* n_saved;
  int* return_code;
  double* seconds;     // [2]: warmup, sampling
  unsigned long long* draws_used;  // [2]: uniforms, normals
  long long* n_grad_total;
} oracle_chain_out;

// Runs num_chains chains (chain ids init_chain_id + i) on num_threads host
// threads, one chain per thread at a time, like the reference's TBB fan-out
// (hmc_nuts_diag_e_adapt.hpp:387-401).
int oracle_sample(void* mp, const oracle_sampler_config* c, int num_chains,
                  const double* inits, const double* inv_metrics, int num_threads,
                  oracle_chain_out* outs) {
  const Model& m = *static_cast<Model*>(mp);
  SamplerConfig cfg;
  cfg.num_warmup = c->num_warmup;
  cfg.num_samples = c->num_samples;
  cfg.num_thin = c->num_thin;
  cfg.save_warmup = c->save_warmup;
  cfg.refresh = c->refresh;
  cfg.stepsize = c->stepsize;
  cfg.stepsize_jitter = c->stepsize_jitter;
  cfg.max_depth = c->max_depth;
  cfg.delta = c->delta;
  cfg.gamma = c->gamma;
  cfg.kappa = c->kappa;
  cfg.t0 = c->t0;
  cfg.init_buffer = c->init_buffer;
  cfg.term_buffer = c->term_buffer;
  cfg.window = c->window;
  cfg.init_radius = c->init_radius;
  cfg.seed = c->seed;
  cfg.init_chain_id = c->init_chain_id;
  cfg.adapt = c->adapt;
  cfg.dense = c->dense;
  const int D = m.D;
  const size_t MD = cfg.dense ? (size_t)D * D : (size_t)D;
  std::atomic<int> next(0);
  auto worker = [&]() {
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= num_chains) break;
      ChainOut o;
      run_chain(m, cfg, inits ? inits + (size_t)i * D : nullptr,
                inv_metrics ? inv_metrics + (size_t)i * MD : nullptr,
                cfg.init_chain_id + (unsigned)i, o);
      oracle_chain_out& dst = outs[i];
      if (dst.rows && !o.rows.empty())
        std::memcpy(dst.rows, o.rows.data(), o.rows.size() * sizeof(double));
      if (dst.unc && !o.unc.empty())
        std::memcpy(dst.unc, o.unc.data(), o.unc.size() * sizeof(double));
      if (dst.init && !o.init.empty())
        std::memcpy(dst.init, o.init.data(), D * sizeof(double));
      if (dst.inv_metric && !o.inv_metric.empty())
        std::memcpy(dst.inv_metric, o.inv_metric.data(), MD * sizeof(double));
      if (dst.stepsize) *dst.stepsize = o.stepsize;
      if (dst.n_grad) *dst.n_grad = o.n_grad;
      if (dst.n_saved) *dst.n_saved = o.n_saved;
      if (dst.return_code) *dst.return_code = o.return_code;
      if (dst.seconds) {
        dst.seconds[0] = o.warm_seconds;
        dst.seconds[1] = o.sample_seconds;
      }
      if (dst.draws_used) {
        dst.draws_used[0] = o.n_uniform;
        dst.draws_used[1] = o.n_normal;
      }
      if (dst.n_grad_total) *dst.n_grad_total = o.n_grad_total;
    }
  };
  int nt = std::max(1, std::min(num_threads, num_chains));
  std::vector<std::thread> ts;
  for (int t = 0; t < nt; ++t) ts.emplace_back(worker);
  for (auto& t : ts) t.join();
  return 0;
}

// --- dual averaging step (stepsize_adaptation.hpp:55-71).  state:
// [counter, s_bar, x_bar, mu, delta, gamma, kappa, t0], updated in place.
void oracle_learn_stepsize(double* state, double* epsilon, double adapt_stat) {
  StepsizeAdaptation a;
  a.counter = state[0];
  a.s_bar = state[1];
  a.x_bar = state[2];
  a.mu = state[3];
  a.delta = state[4];
  a.gamma = state[5];
  a.kappa = state[6];
  a.t0 = state[7];
  a.learn_stepsize(*epsilon, adapt_stat);
  state[0] = a.counter;
  state[1] = a.s_bar;
  state[2] = a.x_bar;
}

// --- window schedule: for each of n_iter learn_variance calls with draws q
// (n_iter x d), out_update[i] = 1 when the metric was updated at call i.
// var_out receives the final variance.  Logger lines are joined by '\n'.
int oracle_var_adaptation(unsigned num_warmup, unsigned init_buffer,
                          unsigned term_buffer, unsigned window, int d,
                          int n_iter, const double* q, double* var_out,
                          int* out_update, char* log_buf, int log_cap) {
  Logger logger;
  VarAdaptation va(d);
  va.set_window_params(num_warmup, init_buffer, term_buffer, window, logger);
  Vec var(var_out, var_out + d);
  try {
    for (int i = 0; i < n_iter; ++i) {
      Vec qi(q + (size_t)i * d, q + (size_t)(i + 1) * d);
      out_update[i] = va.learn_variance(var, qi) ? 1 : 0;
    }
  } catch (const std::exception&) {
    return 1;
  }
  for (int i = 0; i < d; ++i) var_out[i] = var[i];
  std::string joined;
  for (auto& l : logger.lines) joined += l + "\n";
  if (log_buf && log_cap > 0) {
    std::strncpy(log_buf, joined.c_str(), log_cap - 1);
    log_buf[log_cap - 1] = 0;
  }
  return 0;
}

// --- covar_adaptation over n_iter draws q (n_iter x d); covar_out (d x d,
// row-major) holds the starting covariance and receives the result.
int oracle_covar_adaptation(unsigned num_warmup, unsigned init_buffer, unsigned term_buffer,
                            unsigned window, int d, int n_iter, const double* q,
                            double* covar_out, int* out_update) {
  Logger logger;
  CovarAdaptation ca(d);
  ca.set_window_params(num_warmup, init_buffer, term_buffer, window, logger);
  Vec covar(covar_out, covar_out + (size_t)d * d);
  try {
    for (int i = 0; i < n_iter; ++i) {
      Vec qi(q + (size_t)i * d, q + (size_t)(i + 1) * d);
      out_update[i] = ca.learn_covariance(covar, qi) ? 1 : 0;
    }
  } catch (const std::exception&) {
    return 1;
  }
  std::copy(covar.begin(), covar.end(), covar_out);
  return 0;
}

// --- dense_e_metric pieces: T(p) and dtau_dp for inverse metric a (d x d);
// n momenta drawn by sample_p from chain `chain`'s normals; the validation.
// Returns 0, or 1 when a is not a valid inverse metric.
int oracle_dense_metric(int d, const double* a, const double* p, double* T, double* dtau,
                        unsigned seed, unsigned chain, int n, double* draws) {
  Vec av(a, a + (size_t)d * d);
  if (!dense_metric_ok(av, d)) return 1;
  Model dummy;
  DenseEHamiltonian h(dummy, d);
  h.set_metric(av);
  PsPoint z(d);
  if (p) {
    for (int i = 0; i < d; ++i) z.p[i] = p[i];
    if (T) *T = h.T(z);
    if (dtau) {
      Vec t = h.dtau_dp(z);
      std::copy(t.begin(), t.end(), dtau);
    }
  }
  if (draws && n > 0) {
    PhiloxSource rng(seed, chain);
    for (int k = 0; k < n; ++k) {
      h.sample_p(z, rng);
      std::copy(z.p.begin(), z.p.end(), draws + (size_t)k * d);
    }
  }
  return 0;
}

// --- mock sampler scenarios from base_nuts_test.cpp:139-438.
// scenario 1: build_tree_test, 2: rho_aggregation_test, 3: divergence_test,
// 4: transition (mock_nuts), 5: transition_egde_momenta (max_depth 2).
// Uniform draws come from `uniforms`; results are written to out.
// One base_nuts transition (base_nuts.hpp:78-204) of a diag_e sampler from q0
// with scripted draws: uniforms and normals are consumed in the sampler's
// order (sample_p's D normals, then the direction and acceptance uniforms).
// out: q (D values), then lp, accept_stat, depth, n_leapfrog, divergent,
// energy, uniforms used, normals used.  Returns 0, or -1 when the script ran
// out.
int oracle_transition_scripted(void* mp, const double* q0, const double* inv_metric,
                               double stepsize, int max_depth, const double* uniforms, int nu,
                               const double* normals, int nz, double* out) {
  const Model& m = *static_cast<Model*>(mp);
  const int D = m.D;
  try {
    ScriptedSource rng(uniforms, nu, normals, nz);
    DiagEHamiltonian ham(m, D);
    if (inv_metric) ham.inv_metric.assign(inv_metric, inv_metric + D);
    ExplLeapfrog integ;
    Nuts s(ham, integ, rng, D);
    s.set_nominal_stepsize(stepsize);
    s.set_stepsize_jitter(0);
    s.set_max_depth(max_depth);
    Sample init;
    init.q.assign(q0, q0 + D);
    Sample r = s.transition(init);
    for (int i = 0; i < D; ++i) out[i] = r.q[i];
    out[D] = r.log_prob;
    out[D + 1] = r.accept_stat;
    out[D + 2] = s.depth;
    out[D + 3] = s.n_leapfrog;
    out[D + 4] = s.divergent ? 1.0 : 0.0;
    out[D + 5] = s.energy;
    out[D + 6] = (double)rng.n_uniform;
    out[D + 7] = (double)rng.n_normal;
    return 0;
  } catch (const std::exception&) {
    return -1;
  }
}

int oracle_mock_scenario(int scenario, const double* uniforms, int n_uniforms,
                         double* out, int out_cap) {
  try {
    ScriptedSource rng(uniforms, n_uniforms, nullptr, 0);
    const int D = 1;
    const double init_momentum = 1.5;
    int n = 0;
    auto put = [&](double v) {
      if (n < out_cap) out[n] = v;
      ++n;
    };
    if (scenario == 1 || scenario == 2) {
      MockHamiltonian ham;
      MockIntegrator integ;
      MockNuts s(ham, integ, rng, D);
      s.mode = scenario == 2 ? 1 : 0;
      s.set_nominal_stepsize(1);
      s.set_stepsize_jitter(0);
      s.sample_stepsize();
      s.z.q[0] = 0;
      s.z.p[0] = init_momentum;
      PsPoint z_propose(D);
      Vec p_begin(D, 0), p_sharp_begin(D, 0), p_end(D, 0), p_sharp_end(D, 0);
      Vec rho = s.z.p;
      double lsw = -INF, H0 = -0.1, smp = 0;
      int nlf = 0;
      bool valid = s.build_tree(3, z_propose, p_sharp_begin, p_sharp_end, rho,
                                p_begin, p_end, H0, 1, nlf, lsw, smp);
      if (scenario == 1) {
        put(valid);
        put(rho[0]);
        put(p_begin[0]);
        put(p_sharp_begin[0]);
        put(p_end[0]);
        put(p_sharp_end[0]);
        put(s.z.q[0]);
        put(s.z.p[0]);
        put(nlf);
        put(lsw);
        put(smp);
      } else {
        for (double v : s.rho_values) put(v);
      }
    } else if (scenario == 3) {
      DivergentHamiltonian ham;
      ExplLeapfrog integ;
      Nuts s(ham, integ, rng, D);
      s.set_nominal_stepsize(1);
      s.set_stepsize_jitter(0);
      s.sample_stepsize();
      s.z.q[0] = 0;
      s.z.p[0] = init_momentum;
      PsPoint z_propose(D);
      Vec p_begin(D, 0), p_sharp_begin(D, 0), p_end(D, 0), p_sharp_end(D, 0);
      Vec rho = s.z.p;
      double lsw = -INF, H0 = -0.1, smp = 0;
      int nlf = 0;
      const double Vs[3] = {-750, -250, 750};
      for (double v0 : Vs) {
        s.z.V = v0;
        bool valid = s.build_tree(0, z_propose, p_sharp_begin, p_sharp_end, rho,
                                  p_begin, p_end, H0, 1, nlf, lsw, smp);
        put(valid);
        put(s.divergent);
      }
    } else if (scenario == 4 || scenario == 5) {
      MockHamiltonian ham;
      MockIntegrator integ;
      MockNuts s(ham, integ, rng, D);
      s.mode = scenario == 5 ? 2 : 0;
      if (scenario == 5) s.set_max_depth(2);
      s.set_nominal_stepsize(1);
      s.set_stepsize_jitter(0);
      s.sample_stepsize();
      s.z.q[0] = 0;
      s.z.p[0] = init_momentum;
      Sample init;
      init.q = s.z.q;
      // transition() draws no momentum for the mock (sample_p is a no-op), so
      // the state keeps p = 1.5 as in the reference test.
      Sample r = s.transition(init);
      put(s.depth);
      put(s.n_leapfrog);
      put(s.divergent);
      put(r.q[0]);
      put(r.log_prob);
      put(r.accept_stat);
      put((double)rng.n_uniform);
      for (size_t i = 0; i < s.minus_values.size(); ++i) {
        put(s.minus_values[i]);
        put(s.plus_values[i]);
      }
    } else {
      return -1;
    }
    return n;
  } catch (const std::exception&) {
    return -2;
  }
}

}  // extern "C"
