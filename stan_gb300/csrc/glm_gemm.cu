// Batched GLM log density and gradient for wide designs (K + intercept > 128)
// in the bf16 tensor-core forms, as two plain GEMMs around a link kernel:
//
//   eta (N x C, fp32)   = X_bf16 . Theta^T        (cuBLAS bf16 GEMM, fp32 accumulate)
//   link kernel          term, r = d lp / d eta   per (row, chain); lp sums per
//                        chain over row splits; R as bf16 hi (+ lo) parts
//   G   (C x K, fp32)   = R^T . X_bf16            (cuBLAS bf16 GEMM, fp32 accumulate)
//   pack kernel          split partials [1][C][4+K] for the shared finalize
//
// With the hi/lo split (GBNUTS_PREC_BF16X3) Theta, R and (when X is not stored
// in bf16) X are split into bf16 hi + lo parts and the three products hi.hi +
// hi.lo + lo.hi accumulate; the plain form (GBNUTS_PREC_BF16) uses the hi
// parts only.  The GEMMs are plain library contractions; the link, the lp
// reductions and the packing are this file's kernels.  eta and R go through
// device memory (N x C each): the tensor-memory kernel of glm_tct.cu holds
// Theta and the gradient accumulator on chip, which does not fit for K > 127.
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"

namespace gbn {

namespace {

// Row splits of the link kernel: ~128 rows per block (fixed per N: deterministic).
int link_splits(long long N) { return (int)std::max(1LL, std::min(2048LL, N / 128)); }

// X (N x K, any storage type) -> row-major bf16 hi / lo copies with the
// intercept as feature 0, padded to kp features (zeros).
__global__ void gemm_prepare_kernel(const void* X, int x_dtype, long long N, int K, int has_base,
                                    int kp, __nv_bfloat16* xh, __nv_bfloat16* xl) {
  const long long total = N * kp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long row = i / kp;
    const int k = (int)(i - row * kp);
    float v = 0.f;
    if (k < has_base) {
      v = 1.f;
    } else if (k - has_base < K) {
      const long long idx = row * K + (k - has_base);
      if (x_dtype == GBNUTS_F64)
        v = (float)static_cast<const double*>(X)[idx];
      else if (x_dtype == GBNUTS_F32)
        v = static_cast<const float*>(X)[idx];
      else
        v = __uint_as_float(((unsigned)static_cast<const uint16_t*>(X)[idx]) << 16);
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    xh[i] = h;
    if (xl) xl[i] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

// Theta (C x ldq doubles) -> bf16 hi / lo (C x kp); inactive chains get zeros.
__global__ void gemm_theta_kernel(const double* Q, int ldq, int C, const int* active, int kx,
                                  int kp, __nv_bfloat16* th, __nv_bfloat16* tl) {
  const long long total = (long long)C * kp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i / kp);
    const int k = (int)(i - (long long)c * kp);
    const bool act = active == nullptr || active[c] != 0;
    const double d = (act && k < kx) ? Q[(size_t)c * ldq + k] : 0.0;
    const float f = (float)d;
    const __nv_bfloat16 h = __float2bfloat16_rn(f);
    th[i] = h;
    if (tl) tl[i] = __float2bfloat16_rn(f - __bfloat162float(h));
  }
}

// Link on eta (row-major N x C): thread = chain, block = (row split, 128
// chains).  lp_part[s][c] = sum of the link terms of split s's rows (row
// order, compensated fp32 pairs); R hi / lo written in place of eta's layout.
__global__ void __launch_bounds__(128) gemm_link_kernel(const float* eta, const double* y,
                                                        long long N, int C, int link,
                                                        __nv_bfloat16* rh, __nv_bfloat16* rl,
                                                        double* lp_part) {
  const int c = blockIdx.y * 128 + threadIdx.x;
  const int s = blockIdx.x;
  const long long r0 = N * s / gridDim.x, r1 = N * (s + 1) / gridDim.x;
  if (c >= C) return;
  float hi = 0.f, lo = 0.f;
#pragma unroll 4
  for (long long r = r0; r < r1; ++r) {
    const size_t i = (size_t)r * C + c;
    const float e = eta[i];
    const float yv = (float)y[r];
    float term, resid;
    if (link == LINK_LOGIT) {
      const float ex = __expf(-fabsf(e));
      const float d = 1.f + ex;
      const float inv = 1.f / d;
      const float sig = e >= 0.f ? inv : ex * inv;
      term = yv * e - (fmaxf(e, 0.f) + logf(d));
      resid = yv - sig;
    } else {
      const float mu = expf(e);
      term = yv * e - mu;
      resid = yv - mu;
    }
    // two-sum accumulation of the lp terms
    const float t = hi + term;
    const float bp = t - hi;
    lo += (hi - (t - bp)) + (term - bp);
    hi = t;
    const __nv_bfloat16 h = __float2bfloat16_rn(resid);
    rh[i] = h;
    if (rl) rl[i] = __float2bfloat16_rn(resid - __bfloat162float(h));
  }
  lp_part[(size_t)s * C + c] = (double)hi + (double)lo;
}

// Split partials [1][C][NP]: lp (the link splits' sums: 256 strided partial
// sums, then a fixed tree), sum r (intercept column of G), zeros for the
// hierarchical slots, G for the coefficients.  One block of 256 per chain.
__global__ void __launch_bounds__(256) gemm_pack_kernel(const double* lp_part, int n_parts,
                                                        const float* G, int C, int kp,
                                                        int has_base, int K, const int* active,
                                                        double* P, int NP) {
  __shared__ double red[256];
  const int c = blockIdx.x;
  if (c >= C || (active && !active[c])) return;
  double a = 0.0;
  for (int s = threadIdx.x; s < n_parts; s += 256) a += lp_part[(size_t)s * C + c];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  double* dst = P + (size_t)c * NP;
  const float* g = G + (size_t)c * kp;
  for (int j = threadIdx.x; j < NP; j += blockDim.x) {
    double v = 0.0;
    if (j == 0)
      v = red[0];
    else if (j == 1)
      v = has_base ? (double)g[0] : 0.0;
    else if (j >= 4)
      v = (double)g[has_base + (j - 4)];
    dst[j] = v;
  }
}

// Per (model, chain count) device buffers and the cuBLAS handle.
struct GemmWork {
  int C = 0, kp = 0;
  long long N = 0;
  __nv_bfloat16 *th = nullptr, *tl = nullptr, *rh = nullptr, *rl = nullptr;
  float *eta = nullptr, *G = nullptr;
  double* lp_part = nullptr;
  void* cublas_ws = nullptr;
  cublasHandle_t handle = nullptr;
};

constexpr size_t kCublasWorkspace = 32u << 20;

void free_gemm_work(GemmWork* w) {
  if (!w) return;
  cudaFree(w->th);
  cudaFree(w->tl);
  cudaFree(w->rh);
  cudaFree(w->rl);
  cudaFree(w->eta);
  cudaFree(w->G);
  cudaFree(w->lp_part);
  cudaFree(w->cublas_ws);
  if (w->handle) cublasDestroy(w->handle);
  delete w;
}

int gemm_fail(cublasStatus_t st, const char* what) {
  set_last_error(std::string("cuBLAS ") + what + " failed (status " + std::to_string((int)st) + ")");
  return GBNUTS_SOFTWARE;
}

}  // namespace

int gemm_kpad(const ModelDesc& m) { return (m.K + m.has_base + 7) & ~7; }

int gemm_prepare(const ModelDesc& m, void** xh, void** xl, cudaStream_t st) {
  const int kp = gemm_kpad(m);
  const size_t n = (size_t)m.N * kp;
  GBN_CUDA_TRY(cudaMalloc(xh, n * sizeof(__nv_bfloat16)));
  *xl = nullptr;
  if (m.x_dtype != GBNUTS_BF16) GBN_CUDA_TRY(cudaMalloc(xl, n * sizeof(__nv_bfloat16)));
  gemm_prepare_kernel<<<152 * 8, 256, 0, st>>>(m.X, m.x_dtype, m.N, m.K, m.has_base, kp,
                                               static_cast<__nv_bfloat16*>(*xh),
                                               static_cast<__nv_bfloat16*>(*xl));
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

void gemm_free_work(GradWorkspace& ws) {
  free_gemm_work(static_cast<GemmWork*>(ws.gemm));
  ws.gemm = nullptr;
}

int launch_gemm(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
                const int* active, GradWorkspace& ws, cudaStream_t st) {
  const int kp = gemm_kpad(m);
  const int kx = m.K + m.has_base;
  const bool split = precision == GBNUTS_PREC_BF16X3;
  GemmWork* w = static_cast<GemmWork*>(ws.gemm);
  if (w && (w->C != C || w->kp != kp || w->N != m.N)) {
    gemm_free_work(ws);
    w = nullptr;
  }
  if (!w) {
    w = new GemmWork();
    ws.gemm = w;
    w->C = C;
    w->kp = kp;
    w->N = m.N;
    const size_t nc = (size_t)m.N * C;
    GBN_CUDA_TRY(cudaMalloc(&w->th, (size_t)C * kp * sizeof(__nv_bfloat16)));
    GBN_CUDA_TRY(cudaMalloc(&w->tl, (size_t)C * kp * sizeof(__nv_bfloat16)));
    GBN_CUDA_TRY(cudaMalloc(&w->eta, nc * sizeof(float)));
    GBN_CUDA_TRY(cudaMalloc(&w->rh, nc * sizeof(__nv_bfloat16)));
    GBN_CUDA_TRY(cudaMalloc(&w->rl, nc * sizeof(__nv_bfloat16)));
    GBN_CUDA_TRY(cudaMalloc(&w->G, (size_t)C * kp * sizeof(float)));
    GBN_CUDA_TRY(cudaMalloc(&w->lp_part, (size_t)link_splits(m.N) * C * sizeof(double)));
    GBN_CUDA_TRY(cudaMalloc(&w->cublas_ws, kCublasWorkspace));
    cublasStatus_t cs = cublasCreate(&w->handle);
    if (cs != CUBLAS_STATUS_SUCCESS) return gemm_fail(cs, "create");
    cs = cublasSetWorkspace(w->handle, w->cublas_ws, kCublasWorkspace);
    if (cs != CUBLAS_STATUS_SUCCESS) return gemm_fail(cs, "workspace");
  }
  cublasStatus_t cs = cublasSetStream(w->handle, st);
  if (cs != CUBLAS_STATUS_SUCCESS) return gemm_fail(cs, "stream");

  gemm_theta_kernel<<<std::max(1, std::min(152 * 4, (C * kp + 255) / 256)), 256, 0, st>>>(
      Q, ldq, C, active, kx, kp, w->th, split ? w->tl : nullptr);
  GBN_CUDA_TRY(cudaGetLastError());

  const __nv_bfloat16* xh = static_cast<const __nv_bfloat16*>(m.gx_h);
  const __nv_bfloat16* xl = static_cast<const __nv_bfloat16*>(m.gx_l);
  const float one = 1.f, zero = 0.f;
  // eta (column-major C x N) = Theta (C x kp) . X^T (kp x N): products in order
  // hi.hi, hi.lo (Theta lo), lo.hi (X lo).
  struct Prod {
    const __nv_bfloat16 *a, *b;
  };
  Prod fwd[3] = {{w->th, xh}, {w->tl, xh}, {w->th, xl}};
  const int n_fwd = split ? (xl ? 3 : 2) : 1;
  for (int i = 0; i < n_fwd; ++i) {
    cs = cublasGemmEx(w->handle, CUBLAS_OP_T, CUBLAS_OP_N, C, (int)m.N, kp, &one, fwd[i].a,
                      CUDA_R_16BF, kp, fwd[i].b, CUDA_R_16BF, kp, i ? &one : &zero, w->eta,
                      CUDA_R_32F, C, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
    if (cs != CUBLAS_STATUS_SUCCESS) return gemm_fail(cs, "forward GEMM");
  }
  const int nsplit = link_splits(m.N);
  dim3 lgrid(nsplit, (C + 127) / 128);
  gemm_link_kernel<<<lgrid, 128, 0, st>>>(w->eta, m.y, m.N, C, m.link, w->rh,
                                          split ? w->rl : nullptr, w->lp_part);
  GBN_CUDA_TRY(cudaGetLastError());
  // G (column-major kp x C) = X^T (kp x N) . R (N x C): R hi with X hi, R lo
  // with X hi, R hi with X lo.
  Prod adj[3] = {{xh, w->rh}, {xh, w->rl}, {xl, w->rh}};
  for (int i = 0; i < n_fwd; ++i) {
    cs = cublasGemmEx(w->handle, CUBLAS_OP_N, CUBLAS_OP_T, kp, C, (int)m.N, &one, adj[i].a,
                      CUDA_R_16BF, kp, adj[i].b, CUDA_R_16BF, C, i ? &one : &zero, w->G,
                      CUDA_R_32F, kp, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
    if (cs != CUBLAS_STATUS_SUCCESS) return gemm_fail(cs, "adjoint GEMM");
  }
  gemm_pack_kernel<<<C, 256, 0, st>>>(w->lp_part, nsplit, w->G, C, kp, m.has_base, m.K,
                                      active, ws.partial, ws.NP);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

}  // namespace gbn
