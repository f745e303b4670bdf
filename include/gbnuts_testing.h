/*
 * Test hooks of the gbnuts library.  They have no counterpart in the
 * reference; they exist so the tests can check device building blocks in
 * isolation.
 */
#ifndef GBNUTS_TESTING_H
#define GBNUTS_TESTING_H
#include <stdint.h>

#include "gbnuts.h"
#ifdef __cplusplus
extern "C" {
#endif

/* The chains-on-M layouts: D1 = A . X^T and D2 = R . X with A and R held in
 * tensor memory (128 lanes x 64 32-bit words each, Aw / Rw, written as given:
 * two bf16 per word) and X a 128x128 bf16 matrix (row-major uint16 bit
 * patterns); D1, D2 128x128 fp32 outputs.  Returns 0 on success. */
int gbnuts_tct_probe(const uint32_t* Aw, const uint16_t* X, const uint32_t* Rw, float* D1,
                     float* D2);

/* gbnuts_sample_run with every chain's draws taken from the given arrays
 * instead of the counter-based stream: chain c's uniform #n is
 * uniforms[c * n_per_chain + n] and its normal #n normals[c * n_per_chain + n]
 * (NaN past the end), consumed in the sampler's order (initial values,
 * momentum draws, tree directions and acceptances).  For replaying a
 * transition whose draws are known. */
int gbnuts_sample_run_scripted(gbnuts_model* m, const gbnuts_run_config* cfg,
                               gbnuts_run_output* out, const double* uniforms,
                               const double* normals, int n_per_chain);

/* A bounded device wait made to run out: one thread waits on an mbarrier
 * that nothing arrives on, with a limit of limit_cycles SM clock cycles (the
 * library's kernels use about 2 s).  *code receives the error code the wait
 * recorded (0 if it completed), *completed 1 if it completed.  Returns 0 when
 * the launch ran and the device stayed usable. */
int gbnuts_wait_probe(long long limit_cycles, int* code, int* completed);

/* gbnuts_log_prob_grad_batch (propto, with Jacobian) over the points whose
 * active[i] is non-zero, the way a sampler step evaluates the chains that
 * request a gradient: in the narrow tensor-core forms the kernel packs the
 * active points into as few 128-point groups as they fill (its planned
 * launch).  lp and grad of inactive points are unspecified. */
int gbnuts_log_prob_grad_batch_active(gbnuts_model* m, const double* theta, int num_points,
                                      const int* active, int precision, double* lp,
                                      double* grad);

#ifdef __cplusplus
}
#endif
#endif
