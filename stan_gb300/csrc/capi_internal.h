// Internals shared by the host-side translation units (not installed).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"
#include "nuts_device.h"

inline int fail(int code, const std::string& msg) {
  gbn::set_last_error(msg);
  return code;
}

struct gbnuts_model {
  gbn::ModelDesc desc;
  void* d_X = nullptr;
  double* d_y = nullptr;
  int* d_group = nullptr;
  std::vector<int> h_group_off;  // J+1
  // single-point and batch scratch (owned by the handle)
  gbn::GradWorkspace ws;
  double* d_theta = nullptr;
  double* d_lp = nullptr;
  double* d_grad = nullptr;
  int scratch_C = 0;
  cudaStream_t stream = nullptr;
  void* d_tc_xt = nullptr;
  void* d_tc_xt16 = nullptr;
  float* d_tc_yt = nullptr;
  void* d_wide_xt = nullptr;
};


// Validates a run configuration and builds the device sampler configuration
// (service set-up, hmc_nuts_diag_e_adapt.hpp:360-381); messages receive the
// window-schedule warnings of set_window_params.
int make_sampler_cfg(const gbnuts_model* m, const gbnuts_run_config* rc, int max_rows,
                     int out_cols, gbn::SamplerCfg* cfg, std::vector<std::string>* messages);
