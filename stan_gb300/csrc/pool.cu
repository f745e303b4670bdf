// Continuous batching of many posterior fits on one GPU.
//
// Fits arrive (gbnuts_pool_submit) with their data and run configuration and
// wait in a FIFO queue.  Each gbnuts_pool_step call retires fits whose chains
// have all finished (copying their draws to the caller's buffers and freeing
// their device memory), admits queued fits while a slot, the chain budget and
// free device memory allow, and then runs steps in which every chain of every
// admitted fit advances together: one launch of the NUTS state machine over
// the chains of all fits (nuts_step_pool_kernel) and one launch of the
// gradient stage over a work table of (fit, row split, chain block) items
// (loglik_partial_pool_kernel).  Fits of different N, K and J, at different
// points of warmup or sampling and with different tree depths, share those
// launches; a fit admitted later starts in the next step.
//
// A fit's arithmetic does not depend on its neighbours: its row splits and
// tile rows are those a run of the fit alone would use, and every chain's
// state machine only touches its own fit's data, so its draws are the same
// alone and in any mix.
//
// The reference has no counterpart: its service runs one fit per call
// (src/stan/services/sample/hmc_nuts_diag_e_adapt.hpp:331-407).
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace gbn;

namespace {

struct PendingFit {
  long long id = 0;
  int kind = 0, x_dtype = 0, K = 0, J = 0, intercept = 1;
  long long N = 0;
  std::vector<unsigned char> X;
  std::vector<double> y, hp, inits, invm;
  std::vector<int> group;
  gbnuts_run_config rc{};
  gbnuts_run_output* out = nullptr;
  std::chrono::steady_clock::time_point submitted;
};

struct ActiveFit {
  long long id = 0;
  gbnuts_model* model = nullptr;
  SamplerCfg cfg{};
  int C = 0, slot = 0;
  std::vector<void*> allocs;
  ChainState* states = nullptr;
  ChainStack* stacks = nullptr;
  double *vecs = nullptr, *req = nullptr, *draws = nullptr, *diag = nullptr,
         *init_out = nullptr, *inits = nullptr, *invm = nullptr;
  int* active = nullptr;
  double* P = nullptr;
  double* Gz = nullptr;
  long long* split_rows = nullptr;
  int S = 0, NP = 0, rb = 0, cb = 16;
  size_t smem = 0;
  bool memset_gz = false;
  gbnuts_run_output* out = nullptr;
  std::chrono::steady_clock::time_point admitted;

  template <typename T>
  cudaError_t alloc(T** p, size_t n) {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) allocs.push_back(v);
    *p = static_cast<T*>(v);
    return e;
  }
  void release() {
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    if (model) gbnuts_model_destroy(model);
    model = nullptr;
  }
};

// Device bytes a fit needs besides its model data.
size_t fit_state_bytes(const SamplerCfg& cfg, int S, int NP, int J, int max_rows, bool diag) {
  const size_t C = cfg.C;
  size_t b = C * (sizeof(ChainState) + sizeof(ChainStack));
  b += C * cfg.n_slots * cfg.ld * 8 + C * cfg.ld * 8 + C * 4;
  b += C * (size_t)max_rows * cfg.n_cols * 8;
  if (diag) b += C * (size_t)max_rows * 3 * cfg.D * 8;
  b += C * cfg.D * 8 * 3;
  b += (size_t)S * C * NP * 8 + (size_t)(S + 1) * 8 + C * (size_t)J * 8;
  return b;
}

}  // namespace

struct gbnuts_pool {
  int precision = GBNUTS_PREC_FP64, x_dtype = GBNUTS_F32, max_fits = 0;
  long long max_chains = 0;
  long long reserve_bytes = 0;
  cudaStream_t stream = nullptr;
  // side streams and events: launches of different classes (team size, chains
  // per block) of the same step run concurrently
  cudaStream_t side[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[3] = {nullptr, nullptr, nullptr};
  int* d_done = nullptr;
  int* d_abort = nullptr;
  int* h_done = nullptr;  // pinned
  std::deque<PendingFit> queue;
  std::vector<ActiveFit*> active;
  std::vector<int> free_slots;
  std::map<long long, std::pair<int, int>> status;  // id -> (state, return code)
  long long next_id = 1;
  bool dirty = true;
  long long total_chains = 0;
  long long steps = 0;
  // device tables
  PoolFitDev* d_fits = nullptr;
  PoolGradFit* d_gfits = nullptr;
  int2* d_chain_map = nullptr;
  PoolWorkItem* d_items = nullptr;
  size_t cap_fits = 0, cap_gfits = 0, cap_chains = 0, cap_items = 0;
  int n_chain_map = 0, n_items = 0;
  int team_off[4] = {0, 0, 0, 0}, team_n[4] = {0, 0, 0, 0};  // chain map by team size
  int item_off[3] = {0, 0, 0}, item_n[3] = {0, 0, 0};  // work items by chains per block
  size_t smem_cb[3] = {0, 0, 0};
};

enum { POOL_QUEUED = 0, POOL_RUNNING = 1, POOL_DONE = 2, POOL_UNKNOWN = 3 };

static int admit(gbnuts_pool* p, PendingFit& pf, bool force) {
  // model (device copies of X, y, group)
  gbnuts_model* m = nullptr;
  int rc = gbnuts_model_create(pf.kind, pf.X.empty() ? nullptr : pf.X.data(), pf.x_dtype,
                               pf.y.data(), pf.group.empty() ? nullptr : pf.group.data(), pf.N,
                               pf.K, pf.J, pf.intercept, pf.hp.empty() ? nullptr : pf.hp.data(),
                               (int)pf.hp.size(), &m);
  if (rc) return rc;
  ActiveFit* f = new ActiveFit();
  f->model = m;
  f->id = pf.id;
  f->out = pf.out;
  if (!pf.inits.empty() && pf.inits.size() != (size_t)pf.rc.num_chains * m->desc.D) rc = GBNUTS_USAGE;
  if (rc == GBNUTS_OK) {
    gbnuts_run_config rcc = pf.rc;
    rcc.inits = pf.inits.empty() ? nullptr : pf.inits.data();
    rcc.inv_metrics = pf.invm.empty() ? nullptr : pf.invm.data();
    rc = make_sampler_cfg(m, &rcc, pf.out->max_rows, pf.out->n_cols, &f->cfg, nullptr);
  }
  if (rc) {
    f->release();
    delete f;
    return rc;
  }
  const ModelDesc& d = m->desc;
  const int C = f->cfg.C;
  f->C = C;
  f->S = choose_splits(d, C, p->precision);
  f->NP = n_partials(d);
  f->cb = block_chains(d.K, C);
  f->rb = partial_tile_rows(d.K, C, p->precision);
  f->smem = partial_smem(d.K, C, f->rb, p->precision);
  const int J = d.off_z >= 0 ? d.J : 0;
  const size_t need = fit_state_bytes(f->cfg, f->S, f->NP, J, pf.out->max_rows,
                                      pf.out->diagnostics != nullptr);
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  if (!force && (long long)free_b - (long long)need < p->reserve_bytes) {
    f->release();
    delete f;
    return -1;  // not now
  }
  cudaError_t e = cudaSuccess;
  const SamplerCfg& cfg = f->cfg;
  const int mr = pf.out->max_rows;
  if (e == cudaSuccess) e = f->alloc(&f->states, C);
  if (e == cudaSuccess) e = f->alloc(&f->stacks, C);
  if (e == cudaSuccess) e = f->alloc(&f->vecs, (size_t)C * cfg.n_slots * cfg.ld);
  if (e == cudaSuccess) e = f->alloc(&f->req, (size_t)C * cfg.ld);
  if (e == cudaSuccess) e = f->alloc(&f->active, C);
  if (e == cudaSuccess) e = f->alloc(&f->draws, (size_t)C * mr * cfg.n_cols);
  if (e == cudaSuccess && pf.out->diagnostics) e = f->alloc(&f->diag, (size_t)C * mr * 3 * d.D);
  if (e == cudaSuccess) e = f->alloc(&f->init_out, (size_t)C * d.D);
  if (e == cudaSuccess && !pf.inits.empty()) e = f->alloc(&f->inits, pf.inits.size());
  if (e == cudaSuccess && !pf.invm.empty()) e = f->alloc(&f->invm, pf.invm.size());
  if (e == cudaSuccess) e = f->alloc(&f->P, (size_t)f->S * C * f->NP);
  if (e == cudaSuccess) e = f->alloc(&f->split_rows, f->S + 1);
  if (e == cudaSuccess && J > 0) e = f->alloc(&f->Gz, (size_t)C * J);
  if (e != cudaSuccess) {
    f->release();
    delete f;
    cudaGetLastError();
    return force ? fail(GBNUTS_SOFTWARE, "device memory for the fit") : -1;
  }
  std::vector<long long> rows(f->S + 1);
  bool empty_group = false;
  for (int s = 0; s <= f->S; ++s)
    rows[s] = J > 0 ? m->h_group_off[(long long)J * s / f->S] : d.N * s / f->S;
  for (int j = 0; j < J; ++j)
    if (m->h_group_off[j + 1] == m->h_group_off[j]) empty_group = true;
  f->memset_gz = empty_group;
  cudaStream_t st = p->stream;
  e = cudaMemcpyAsync(f->split_rows, rows.data(), rows.size() * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && f->inits)
    e = cudaMemcpyAsync(f->inits, pf.inits.data(), pf.inits.size() * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && f->invm)
    e = cudaMemcpyAsync(f->invm, pf.invm.data(), pf.invm.size() * 8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(f->draws, 0, (size_t)C * mr * cfg.n_cols * 8, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(f->req, 0, (size_t)C * cfg.ld * 8, st);
  if (e == cudaSuccess && f->Gz) e = cudaMemsetAsync(f->Gz, 0, (size_t)C * J * 8, st);
  if (e == cudaSuccess) {
    f->slot = p->free_slots.back();
    p->free_slots.pop_back();
    e = cudaMemsetAsync(p->d_done + f->slot, 0, sizeof(int), st);
  }
  if (e != cudaSuccess) {
    f->release();
    delete f;
    return fail(GBNUTS_SOFTWARE, std::string("fit set-up: ") + cudaGetErrorString(e));
  }
  launch_nuts_init(cfg, f->states, f->stacks, f->vecs, f->invm, f->active, st);
  f->admitted = std::chrono::steady_clock::now();
  p->active.push_back(f);
  p->total_chains += C;
  p->status[f->id] = {POOL_RUNNING, 0};
  p->dirty = true;
  return GBNUTS_OK;
}

// Copies a finished fit's results to the caller's buffers and frees it.
static int retire(gbnuts_pool* p, ActiveFit* f) {
  const SamplerCfg& cfg = f->cfg;
  const int C = f->C, D = cfg.D;
  gbnuts_run_output* out = f->out;
  std::vector<ChainState> hs(C);
  int rc = GBNUTS_OK;
  cudaError_t e = cudaMemcpy(hs.data(), f->states, C * sizeof(ChainState), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(out->draws, f->draws, (size_t)C * out->max_rows * cfg.n_cols * 8,
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && out->diagnostics && f->diag)
    e = cudaMemcpy(out->diagnostics, f->diag, (size_t)C * out->max_rows * 3 * D * 8,
                   cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && out->init)
    e = cudaMemcpy(out->init, f->init_out, (size_t)C * D * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && out->inv_metric)
    e = cudaMemcpy2D(out->inv_metric, D * 8, f->vecs + (size_t)SL_INVM * cfg.ld,
                     (size_t)cfg.n_slots * cfg.ld * 8, D * 8, C, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = fail(GBNUTS_SOFTWARE, std::string("fit readback: ") + cudaGetErrorString(e));
  if (rc == GBNUTS_OK && (out->ess || out->summary)) {
    // convergence report on the device, before the fit's memory is freed
    int w = 0, nr = out->max_rows;
    for (int c = 0; c < C; ++c) {
      w = std::max(w, hs[c].warm_rows);
      nr = std::min(nr, hs[c].rows);
    }
    rc = fit_ess(f->draws, C, out->max_rows, cfg.n_cols, w, std::max(0, nr - w), out->ess,
                 out->summary, p->stream);
  }
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - f->admitted).count();
  for (int c = 0; c < C && rc == GBNUTS_OK; ++c) {
    out->n_rows[c] = hs[c].rows;
    if (out->n_warmup_rows) out->n_warmup_rows[c] = hs[c].warm_rows;
    if (out->status) out->status[c] = hs[c].status;
    if (out->stepsize) out->stepsize[c] = hs[c].nom_eps;
    if (out->n_grad) out->n_grad[c] = hs[c].n_grad;
    if (out->seconds) {
      const double frac = (hs[c].warm_end_ngrad >= 0 && hs[c].n_grad > 0)
                              ? (double)hs[c].warm_end_ngrad / (double)hs[c].n_grad
                              : 0.0;
      out->seconds[2 * c] = wall * frac;
      out->seconds[2 * c + 1] = wall * (1.0 - frac);
    }
    if (hs[c].status == GBNUTS_CHAIN_INIT_FAILED || hs[c].status == GBNUTS_CHAIN_BAD_METRIC)
      rc = GBNUTS_CONFIG;
    else if (hs[c].status != GBNUTS_CHAIN_OK && hs[c].status != GBNUTS_CHAIN_STEPSIZE_INIT_FAILED)
      rc = GBNUTS_SOFTWARE;
  }
  out->total_ms = wall * 1e3;
  p->status[f->id] = {POOL_DONE, rc};
  p->free_slots.push_back(f->slot);
  p->total_chains -= C;
  f->release();
  delete f;
  p->dirty = true;
  return GBNUTS_OK;
}

template <typename T>
static cudaError_t grow(T** buf, size_t* cap, size_t need) {
  if (need <= *cap) return cudaSuccess;
  if (*buf) cudaFree(*buf);
  size_t n = std::max<size_t>(need, *cap * 2 + 16);
  cudaError_t e = cudaMalloc(buf, n * sizeof(T));
  *cap = e == cudaSuccess ? n : 0;
  return e;
}

static int rebuild_tables(gbnuts_pool* p) {
  std::vector<PoolFitDev> fits;
  std::vector<PoolGradFit> gfits;
  std::vector<int2> cmap_team[4];  // chains by team size 1, 2, 4, 8 warps
  std::vector<PoolWorkItem> items_cb[3];  // work items by chains per block 4, 8, 16
  size_t smem_cb[3] = {0, 0, 0};
  for (size_t i = 0; i < p->active.size(); ++i) {
    ActiveFit* f = p->active[i];
    PoolFitDev pf;
    pf.cfg = f->cfg;
    pf.m = f->model->desc;
    pf.f = FitPtrs{f->states, f->stacks, f->vecs, f->req,
                   PartialsView{f->P, f->NP, f->S, f->Gz, nullptr},
                   f->active, f->draws, f->diag, f->init_out, f->inits,
                   p->d_done + f->slot, p->d_abort + f->slot};
    fits.push_back(pf);
    PoolGradFit g;
    g.m = f->model->desc;
    g.Q = f->req;
    g.ldq = f->cfg.ld;
    g.C = f->C;
    g.active = f->active;
    g.split_rows = f->split_rows;
    g.P = f->P;
    g.NP = f->NP;
    g.Gz = f->Gz;
    gfits.push_back(g);
    const int tw = team_warps(f->cfg.D);
    for (int c = 0; c < f->C; ++c)
      cmap_team[tw == 1 ? 0 : (tw == 2 ? 1 : (tw == 4 ? 2 : 3))].push_back(make_int2((int)i, c));
    const int kc = f->cb == 4 ? 0 : (f->cb == 8 ? 1 : 2);
    const int blocks = (f->C + f->cb - 1) / f->cb;
    for (int s = 0; s < f->S; ++s)
      for (int b = 0; b < blocks; ++b) items_cb[kc].push_back(PoolWorkItem{(int)i, s, b, f->rb});
    smem_cb[kc] = std::max(smem_cb[kc], f->smem);
  }
  std::vector<PoolWorkItem> items;
  for (int k = 0; k < 3; ++k) {
    p->item_off[k] = (int)items.size();
    p->item_n[k] = (int)items_cb[k].size();
    p->smem_cb[k] = smem_cb[k];
    items.insert(items.end(), items_cb[k].begin(), items_cb[k].end());
  }
  std::vector<int2> cmap;
  for (int k = 0; k < 4; ++k) {
    p->team_off[k] = (int)cmap.size();
    p->team_n[k] = (int)cmap_team[k].size();
    cmap.insert(cmap.end(), cmap_team[k].begin(), cmap_team[k].end());
  }
  cudaError_t e = grow(&p->d_fits, &p->cap_fits, fits.size());
  if (e == cudaSuccess) e = grow(&p->d_gfits, &p->cap_gfits, gfits.size());
  if (e == cudaSuccess) e = grow(&p->d_chain_map, &p->cap_chains, cmap.size());
  if (e == cudaSuccess) e = grow(&p->d_items, &p->cap_items, items.size());
  if (e == cudaSuccess && !fits.empty())
    e = cudaMemcpyAsync(p->d_fits, fits.data(), fits.size() * sizeof(PoolFitDev),
                        cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess && !gfits.empty())
    e = cudaMemcpyAsync(p->d_gfits, gfits.data(), gfits.size() * sizeof(PoolGradFit),
                        cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess && !cmap.empty())
    e = cudaMemcpyAsync(p->d_chain_map, cmap.data(), cmap.size() * sizeof(int2),
                        cudaMemcpyHostToDevice, p->stream);
  if (e == cudaSuccess && !items.empty())
    e = cudaMemcpyAsync(p->d_items, items.data(), items.size() * sizeof(PoolWorkItem),
                        cudaMemcpyHostToDevice, p->stream);
  // the host vectors must outlive the copies
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
  if (e != cudaSuccess) return fail(GBNUTS_SOFTWARE, std::string("pool tables: ") + cudaGetErrorString(e));
  p->n_chain_map = (int)cmap.size();
  p->n_items = (int)items.size();
  p->dirty = false;
  return GBNUTS_OK;
}

extern "C" {

int gbnuts_pool_create(int precision, int x_dtype, int max_fits, long long max_chains,
                       long long reserve_bytes, gbnuts_pool** out) {
  if (!out) return fail(GBNUTS_USAGE, "out is NULL");
  *out = nullptr;
  if (precision != GBNUTS_PREC_FP64 && precision != GBNUTS_PREC_FP32)
    return fail(GBNUTS_USAGE, "the pool runs the fp64 and fp32 forms");
  if (x_dtype < GBNUTS_F64 || x_dtype > GBNUTS_BF16) return fail(GBNUTS_USAGE, "unknown x_dtype");
  if (max_fits <= 0 || max_chains <= 0) return fail(GBNUTS_USAGE, "max_fits and max_chains must be positive");
  gbnuts_pool* p = new gbnuts_pool();
  p->precision = precision;
  p->x_dtype = x_dtype;
  p->max_fits = max_fits;
  p->max_chains = max_chains;
  p->reserve_bytes = reserve_bytes;
  cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
    e = cudaStreamCreateWithFlags(&p->side[i], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_join[i], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_done, max_fits * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_abort, max_fits * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p->d_abort, 0, max_fits * sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost(&p->h_done, max_fits * sizeof(int));
  if (e != cudaSuccess) {
    gbnuts_pool_destroy(p);
    return fail(GBNUTS_SOFTWARE, std::string("pool set-up: ") + cudaGetErrorString(e));
  }
  for (int s = max_fits - 1; s >= 0; --s) p->free_slots.push_back(s);
  *out = p;
  return GBNUTS_OK;
}

void gbnuts_pool_destroy(gbnuts_pool* p) {
  if (!p) return;
  if (p->stream) cudaStreamSynchronize(p->stream);
  for (ActiveFit* f : p->active) {
    f->release();
    delete f;
  }
  if (p->d_fits) cudaFree(p->d_fits);
  if (p->d_gfits) cudaFree(p->d_gfits);
  if (p->d_chain_map) cudaFree(p->d_chain_map);
  if (p->d_items) cudaFree(p->d_items);
  if (p->d_done) cudaFree(p->d_done);
  if (p->d_abort) cudaFree(p->d_abort);
  if (p->h_done) cudaFreeHost(p->h_done);
  for (int i = 0; i < 3; ++i) {
    if (p->side[i]) cudaStreamDestroy(p->side[i]);
    if (p->ev_join[i]) cudaEventDestroy(p->ev_join[i]);
  }
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

int gbnuts_pool_submit(gbnuts_pool* p, int kind, const void* X, int x_dtype, const double* y,
                       const int* group, long long N, int K, int J, int intercept,
                       const double* hp, int n_hp, const gbnuts_run_config* rc,
                       gbnuts_run_output* out, long long* fit_id) {
  if (!p || !rc || !out || !fit_id || !y || N <= 0 || K < 0)
    return fail(GBNUTS_USAGE, "bad arguments");
  if (x_dtype != p->x_dtype) return fail(GBNUTS_USAGE, "x_dtype differs from the pool's");
  if (chains_per_block(K) == 0) return fail(GBNUTS_USAGE, "K above 2048 is not supported");
  if (rc->num_chains <= 0 || rc->num_chains > p->max_chains)
    return fail(GBNUTS_USAGE, "num_chains must be in 1..max_chains");
  if (!out->draws || !out->n_rows) return fail(GBNUTS_USAGE, "draws / n_rows buffers missing");
  if (rc->metric != GBNUTS_METRIC_DIAG)
    return fail(GBNUTS_USAGE, "the pool runs diag_e fits (dense_e runs through gbnuts_sample_run)");
  PendingFit pf;
  pf.id = p->next_id++;
  pf.kind = kind;
  pf.x_dtype = x_dtype;
  pf.K = K;
  pf.J = J;
  pf.N = N;
  pf.intercept = intercept;
  const size_t xb = (size_t)N * K * (x_dtype == GBNUTS_F64 ? 8 : x_dtype == GBNUTS_F32 ? 4 : 2);
  if (xb) pf.X.assign(static_cast<const unsigned char*>(X), static_cast<const unsigned char*>(X) + xb);
  pf.y.assign(y, y + N);
  if (group) pf.group.assign(group, group + N);
  if (hp && n_hp > 0) pf.hp.assign(hp, hp + n_hp);
  pf.rc = *rc;
  const size_t D = (kind == GBNUTS_HIER_NORMAL)     ? 3 + (size_t)J + K
                   : (kind == GBNUTS_HIER_LOGISTIC) ? 2 + (size_t)J + K
                                                    : (size_t)K + (intercept ? 1 : 0);
  const size_t CD = (size_t)rc->num_chains * D;
  if (rc->inits) pf.inits.assign(rc->inits, rc->inits + CD);
  if (rc->inv_metrics) pf.invm.assign(rc->inv_metrics, rc->inv_metrics + CD);
  pf.rc.inits = nullptr;
  pf.rc.inv_metrics = nullptr;
  pf.out = out;
  pf.submitted = std::chrono::steady_clock::now();
  *fit_id = pf.id;
  p->status[pf.id] = {POOL_QUEUED, 0};
  p->queue.push_back(std::move(pf));
  return GBNUTS_OK;
}

// Retires finished fits, admits queued ones, then runs n_steps steps of every
// admitted fit.  n_running / n_queued (may be NULL) report the state after.
int gbnuts_pool_step(gbnuts_pool* p, int n_steps, int* n_running, int* n_queued) {
  if (!p || n_steps < 0) return fail(GBNUTS_USAGE, "bad arguments");
  // admission: FIFO while a slot, the chain budget and device memory allow
  while (!p->queue.empty() && !p->free_slots.empty()) {
    PendingFit& pf = p->queue.front();
    if (p->total_chains + pf.rc.num_chains > p->max_chains) break;
    const bool force = p->active.empty();
    int rc = admit(p, pf, force);
    if (rc == -1) break;  // not enough free memory now
    if (rc != GBNUTS_OK) p->status[pf.id] = {POOL_DONE, rc};
    p->queue.pop_front();
  }
  if (p->dirty) {
    int rc = rebuild_tables(p);
    if (rc) return rc;
  }
  if (!p->active.empty() && n_steps > 0) {
    // Launches of the present classes: the first on the pool's stream, the
    // others on side streams forked from it and joined back.
    auto classes = [&](const int* counts, int n_classes, auto&& launch) -> int {
      int present = 0;
      for (int k = 0; k < n_classes; ++k) present += counts[k] > 0;
      bool first = true;
      int side = 0;
      if (present > 1) cudaEventRecord(p->ev_fork, p->stream);
      for (int k = 0; k < n_classes; ++k) {
        if (counts[k] == 0) continue;
        cudaStream_t st = p->stream;
        if (!first) {
          st = p->side[side];
          cudaStreamWaitEvent(st, p->ev_fork, 0);
        }
        const int rc = launch(k, st);
        if (rc) return rc;
        if (!first) cudaEventRecord(p->ev_join[side++], st);
        first = false;
      }
      for (int i = 0; i < side; ++i) cudaStreamWaitEvent(p->stream, p->ev_join[i], 0);
      return GBNUTS_OK;
    };
    for (int k = 0; k < n_steps; ++k) {
      classes(p->team_n, 4, [&](int c, cudaStream_t st) {
        launch_nuts_step_pool(p->d_fits, p->d_chain_map + p->team_off[c], p->team_n[c], 1 << c,
                              st);
        return GBNUTS_OK;
      });
      for (ActiveFit* f : p->active)
        if (f->memset_gz)
          cudaMemsetAsync(f->Gz, 0, (size_t)f->C * f->model->desc.J * 8, p->stream);
      const int rc = classes(p->item_n, 3, [&](int c, cudaStream_t st) {
        return launch_partials_pool(p->d_gfits, p->d_items + p->item_off[c], p->item_n[c],
                                    4 << c, p->x_dtype, p->precision, p->smem_cb[c], st);
      });
      if (rc) return rc;
    }
    p->steps += n_steps;
    cudaError_t e = cudaMemcpyAsync(p->h_done, p->d_done, p->max_fits * sizeof(int),
                                    cudaMemcpyDeviceToHost, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return fail(GBNUTS_SOFTWARE, std::string("pool step: ") + cudaGetErrorString(e));
    std::vector<ActiveFit*> keep;
    for (ActiveFit* f : p->active) {
      if (p->h_done[f->slot] >= f->C) {
        int rc = retire(p, f);
        if (rc) return rc;
      } else {
        keep.push_back(f);
      }
    }
    p->active.swap(keep);
  }
  if (n_running) *n_running = (int)p->active.size();
  if (n_queued) *n_queued = (int)p->queue.size();
  return GBNUTS_OK;
}

// state: 0 queued, 1 running, 2 done (return code in *rc), 3 unknown id.
int gbnuts_pool_status(gbnuts_pool* p, long long fit_id, int* state, int* rc) {
  if (!p || !state) return fail(GBNUTS_USAGE, "bad arguments");
  auto it = p->status.find(fit_id);
  if (it == p->status.end()) {
    *state = POOL_UNKNOWN;
    if (rc) *rc = 0;
    return GBNUTS_OK;
  }
  *state = it->second.first;
  if (rc) *rc = it->second.second;
  return GBNUTS_OK;
}

// Steps run so far, chains admitted now.
int gbnuts_pool_stats(gbnuts_pool* p, long long* steps, long long* chains) {
  if (!p) return fail(GBNUTS_USAGE, "bad arguments");
  if (steps) *steps = p->steps;
  if (chains) *chains = p->total_chains;
  return GBNUTS_OK;
}

}  // extern "C"
