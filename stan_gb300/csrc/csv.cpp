// Stan CSV and JSON metric files through the service callbacks: the file
// writers an interface attaches to the sampler's writers.
//
// Row and message format of the reference's writers (paths relative to the
// stan-dev/stan tree):
//   src/stan/callbacks/stream_writer.hpp:16-103 and unique_stream_writer.hpp:
//     names and values comma-separated, one row per call, values through
//     operator<< on a stream of precision sig_figs (printf %.*g); a message is
//     the comment prefix then the message; a blank is the prefix alone
//   src/stan/callbacks/json_writer.hpp:27-230: the metric record
//     {"stepsize", "metric_type", "inv_metric"} written by
//     src/stan/mcmc/hmc/base_hmc.hpp:70-76, with the writer's separators and
//     indentation and NaN / Inf / -Inf for non-finite values
//
// One sample file (and optionally one diagnostic and one metric file) per
// chain.  Rows of one chain are appended to that chain's buffer and written in
// large blocks; different chains touch disjoint state, so the service may call
// the writers of different chains from different threads at once (as the
// reference's per-chain TBB tasks do).
#include <charconv>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"

struct gbnuts_csv {
  struct File {
    FILE* f = nullptr;
    std::string buf;
    bool failed = false;
  };
  int C = 0;
  int chain_id0 = 1;
  int sig_figs = 6;
  std::string prefix;  // comment prefix
  std::vector<File> sample, diag;
  std::string metric_prefix;
  std::vector<int> metric_failed;
};

namespace {

constexpr size_t kFlushBytes = 1 << 20;

void flush(gbnuts_csv::File& f) {
  if (!f.f || f.buf.empty()) return;
  if (fwrite(f.buf.data(), 1, f.buf.size(), f.f) != f.buf.size()) f.failed = true;
  f.buf.clear();
}

// operator<< of a double on a stream of precision p with default flags
// (the %.*g conversion): shortest of fixed / scientific with p significant
// digits, trailing zeros removed
void append_value(std::string& s, double v, int p) {
  char tmp[64];
  const auto r = std::to_chars(tmp, tmp + sizeof(tmp), v, std::chars_format::general, p);
  s.append(tmp, r.ptr);
}

// json_writer::write_value: NaN / Inf / -Inf, else operator<<
void append_json_value(std::string& s, double v, int p) {
  if (v != v)
    s += "NaN";
  else if (v == __builtin_inf())
    s += "Inf";
  else if (v == -__builtin_inf())
    s += "-Inf";
  else
    append_value(s, v, p);
}

gbnuts_csv::File* file_of(void* ctx, int chain, int writer) {
  auto* w = static_cast<gbnuts_csv*>(ctx);
  if (chain < 0 || chain >= w->C) return nullptr;
  std::vector<gbnuts_csv::File>* v = writer == GBNUTS_SAMPLE_WRITER       ? &w->sample
                                     : writer == GBNUTS_DIAGNOSTIC_WRITER ? &w->diag
                                                                          : nullptr;
  if (!v || v->empty() || !(*v)[chain].f) return nullptr;
  return &(*v)[chain];
}

void csv_names(void* ctx, int chain, int writer, const char* const* names, int n) {
  auto* f = file_of(ctx, chain, writer);
  if (!f || n <= 0) return;
  for (int i = 0; i < n; ++i) {
    f->buf += names[i];
    f->buf += i + 1 < n ? ',' : '\n';
  }
  if (f->buf.size() >= kFlushBytes) flush(*f);
}

void csv_values(void* ctx, int chain, int writer, const double* v, int n) {
  auto* f = file_of(ctx, chain, writer);
  if (!f || n <= 0) return;
  const int p = static_cast<gbnuts_csv*>(ctx)->sig_figs;
  for (int i = 0; i < n; ++i) {
    append_value(f->buf, v[i], p);
    f->buf += i + 1 < n ? ',' : '\n';
  }
  if (f->buf.size() >= kFlushBytes) flush(*f);
}

void csv_message(void* ctx, int chain, int writer, const char* msg) {
  auto* f = file_of(ctx, chain, writer);
  if (!f) return;
  f->buf += static_cast<gbnuts_csv*>(ctx)->prefix;
  f->buf += msg;
  f->buf += '\n';
}

void csv_blank(void* ctx, int chain, int writer) {
  auto* f = file_of(ctx, chain, writer);
  if (!f) return;
  f->buf += static_cast<gbnuts_csv*>(ctx)->prefix;
  f->buf += '\n';
}

void csv_metric(void* ctx, int chain, double stepsize, const char* metric_type,
                const double* inv, int n) {
  auto* w = static_cast<gbnuts_csv*>(ctx);
  if (chain < 0 || chain >= w->C || w->metric_prefix.empty()) return;
  // begin_record / write x 3 / end_record of json_writer
  std::string s = "\n{\n  \"stepsize\" : ";
  append_json_value(s, stepsize, w->sig_figs);
  s += ",\n  \"metric_type\" : \"";
  s += metric_type;
  s += "\",\n  \"inv_metric\" : ";
  // a vector, or for dense_e (n = D * D, row-major) json_writer's matrix:
  // the rows as vectors inside one more bracket
  auto vec = [&](const double* v, int len) {
    s += "[ ";
    for (int i = 0; i < len; ++i) {
      append_json_value(s, v[i], w->sig_figs);
      if (i + 1 < len) s += ", ";
    }
    s += " ]";
  };
  if (strcmp(metric_type, "dense_e") == 0) {
    int d = 0;
    while ((long long)(d + 1) * (d + 1) <= n) ++d;
    s += "[ ";
    for (int r = 0; r < d; ++r) {
      vec(inv + (size_t)r * d, d);
      if (r + 1 < d) s += ", ";
    }
    s += " ]";
  } else {
    vec(inv, n);
  }
  s += "\n}\n";
  const std::string path = w->metric_prefix + "_" + std::to_string(w->chain_id0 + chain) +
                           ".json";
  FILE* f = fopen(path.c_str(), "wb");
  if (!f || fwrite(s.data(), 1, s.size(), f) != s.size()) w->metric_failed[chain] = 1;
  if (f && fclose(f) != 0) w->metric_failed[chain] = 1;
}

void close_files(std::vector<gbnuts_csv::File>& v, bool& failed) {
  for (auto& f : v) {
    if (!f.f) continue;
    flush(f);
    if (fclose(f.f) != 0) f.failed = true;
    f.f = nullptr;
    failed |= f.failed;
  }
}

}  // namespace

extern "C" int gbnuts_csv_open(const char* sample_prefix, const char* diagnostic_prefix,
                               const char* metric_prefix, int num_chains, int chain_id0,
                               int sig_figs, gbnuts_callbacks* cb, gbnuts_csv** out) {
  using gbn::set_last_error;
  if (!sample_prefix || !cb || !out || num_chains <= 0 || sig_figs < 1 || sig_figs > 18) {
    set_last_error("gbnuts_csv_open: bad arguments");
    return GBNUTS_USAGE;
  }
  auto* w = new gbnuts_csv;
  w->C = num_chains;
  w->chain_id0 = chain_id0;
  w->sig_figs = sig_figs;
  w->prefix = "# ";
  w->sample.resize(num_chains);
  if (diagnostic_prefix) w->diag.resize(num_chains);
  if (metric_prefix) w->metric_prefix = metric_prefix;
  w->metric_failed.assign(num_chains, 0);
  auto open_all = [&](std::vector<gbnuts_csv::File>& v, const char* pre) {
    for (int c = 0; c < (int)v.size(); ++c) {
      const std::string path = std::string(pre) + "_" + std::to_string(chain_id0 + c) + ".csv";
      v[c].f = fopen(path.c_str(), "wb");
      if (!v[c].f) {
        set_last_error("gbnuts_csv_open: cannot open " + path);
        return false;
      }
    }
    return true;
  };
  if (!open_all(w->sample, sample_prefix) ||
      (diagnostic_prefix && !open_all(w->diag, diagnostic_prefix))) {
    bool f = false;
    close_files(w->sample, f);
    close_files(w->diag, f);
    delete w;
    return GBNUTS_NOINPUT;
  }
  memset(cb, 0, sizeof(*cb));
  cb->ctx = w;
  cb->write_names = csv_names;
  cb->write_values = csv_values;
  cb->write_message = csv_message;
  cb->write_blank = csv_blank;
  cb->write_metric = metric_prefix ? csv_metric : nullptr;
  cb->want_diagnostics = diagnostic_prefix ? 1 : 0;
  cb->chains_concurrent = 1;
  *out = w;
  return GBNUTS_OK;
}

extern "C" int gbnuts_csv_close(gbnuts_csv* w) {
  if (!w) return GBNUTS_OK;
  bool failed = false;
  close_files(w->sample, failed);
  close_files(w->diag, failed);
  for (int x : w->metric_failed) failed |= x != 0;
  delete w;
  if (failed) {
    gbn::set_last_error("gbnuts_csv_close: a write failed");
    return GBNUTS_SOFTWARE;
  }
  return GBNUTS_OK;
}
