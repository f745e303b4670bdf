// Batched GLM log density and gradient on the tcgen05 tensor cores
// (precision GBNUTS_PREC_BF16X3), for the logistic and Poisson families.
//
// For a CTA owning 64 chains and a range of 128-row tiles of X:
//   GEMM1  eta (128 rows x 64 chains)   = X_tile . Theta^T        (TMEM, fp32)
//   link   term, r = d lp / d eta       per (row, chain), fp32, from TMEM
//   GEMM2  G   (128 features x 64 chains) += X_tile^T . R          (TMEM, fp32)
// with X, Theta and R each split into bf16 hi + lo parts and the three
// products hi.hi + hi.lo + lo.hi accumulated in fp32 (x has no lo part when
// it is stored in bf16).  The intercept is feature 0 of the tile (a column
// of ones).  X is pre-tiled once per model into the canonical K-major
// no-swizzle layout (contiguous 32 KiB per tile and part), so a tile is one
// contiguous copy.  The per-chain lp sum over rows is a warp transpose
// reduction of the link terms.  Results go to the same split partials as the
// CUDA-core kernels, so the finalize kernel (priors, split sums) is shared.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"
#include "tc_common.cuh"

namespace gbn {

using namespace tc;

constexpr int TM = 128;   // rows per tile
constexpr int TK = 128;   // features per tile (K + intercept, zero padded)
constexpr int NC = 64;    // chains per CTA
constexpr int TILE_BYTES = TM * TK * 2;      // one bf16 part of an X tile
constexpr int THETA_BYTES = NC * TK * 2;     // one bf16 part of Theta
constexpr int R_BYTES = NC * TM * 2;         // one bf16 part of R
constexpr int SMEM_X = 0;
constexpr int SMEM_T = SMEM_X + 2 * TILE_BYTES;
constexpr int SMEM_R = SMEM_T + 2 * THETA_BYTES;
constexpr int SMEM_LP = SMEM_R + 2 * R_BYTES;
constexpr int SMEM_BAR = SMEM_LP + 4 * NC * 4;
constexpr int SMEM_TOTAL = SMEM_BAR + 64;
constexpr int SMEM_ALLOC = SMEM_TOTAL + 1024;  // slack for 1 KiB alignment

int tc_max_features() { return TK; }

// X tiles: part 0 (hi) and 1 (lo) of tile t at xt + (2t + part) * TM*TK.
__global__ void tc_prepare_tiles_kernel(const void* X, int x_dtype, long long N, int K,
                                        int has_base, int n_tiles, __nv_bfloat16* xt,
                                        const double* y, float* yt) {
  const long long total = (long long)n_tiles * TM * TK;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long t = i / (TM * TK);
    const int e = (int)(i - t * (TM * TK));
    const int r = e / TK, k = e - r * TK;
    const long long row = t * TM + r;
    float v = 0.f;
    if (row < N) {
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
    }
    __nv_bfloat16 hi, lo;
    split_bf16(v, hi, lo);
    const uint32_t off = kmajor_off(r, k, TK) / 2;
    xt[(2 * t) * (TM * TK) + off] = hi;
    xt[(2 * t + 1) * (TM * TK) + off] = lo;
    if (k == 0) yt[t * TM + r] = row < N ? (float)y[row] : 0.f;
  }
}

struct TcArgs {
  const __nv_bfloat16* xt;  // pre-tiled X (hi/lo)
  const float* yt;          // y per tile row
  long long N;
  int K, has_base, n_tiles, link, x_has_lo;
  const double* Q;
  int ldq, C;
  const int* active;
  double* P;
  int NP, S;
  int* err;
};

// Warp transpose reduction: v[64] per lane (one row each) -> lane l holds the
// sums over the warp's 32 rows of chains 2l and 2l+1.
__device__ __forceinline__ void warp_reduce_scatter64(float (&v)[64], float& s0, float& s1) {
  const int lane = threadIdx.x & 31;
  float w[32];
  {
    const bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      float send = up ? v[i] : v[32 + i];
      float keep = up ? v[32 + i] : v[i];
      w[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
  }
  float x[16];
  {
    const bool up = lane & 8;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      float send = up ? w[i] : w[16 + i];
      float keep = up ? w[16 + i] : w[i];
      x[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
  }
  float y[8];
  {
    const bool up = lane & 4;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float send = up ? x[i] : x[8 + i];
      float keep = up ? x[8 + i] : x[i];
      y[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
  }
  float z[4];
  {
    const bool up = lane & 2;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float send = up ? y[i] : y[4 + i];
      float keep = up ? y[4 + i] : y[i];
      z[i] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
  }
  {
    const bool up = lane & 1;
    float send0 = up ? z[0] : z[2], keep0 = up ? z[2] : z[0];
    float send1 = up ? z[1] : z[3], keep1 = up ? z[3] : z[1];
    s0 = keep0 + __shfl_xor_sync(0xffffffffu, send0, 1);
    s1 = keep1 + __shfl_xor_sync(0xffffffffu, send1, 1);
  }
}

__global__ void __launch_bounds__(128, 1) glm_tc_kernel(TcArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char* sXh = sm + SMEM_X;
  unsigned char* sXl = sXh + TILE_BYTES;
  unsigned char* sTh = sm + SMEM_T;
  unsigned char* sTl = sTh + THETA_BYTES;
  unsigned char* sRh = sm + SMEM_R;
  unsigned char* sRl = sRh + R_BYTES;
  float* sLP = reinterpret_cast<float*>(sm + SMEM_LP);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + SMEM_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SMEM_BAR + 16);
  __shared__ int act_s[NC];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s = blockIdx.x;
  const int c0 = blockIdx.y * NC;
  const int hb = a.has_base;
  const int Kx = a.K + hb;

  if (tid < NC) {
    const int cg = c0 + tid;
    act_s[tid] = (cg < a.C) && (a.active == nullptr || a.active[cg] != 0);
  }
  const int any = __syncthreads_or(tid < NC ? act_s[tid] : 0);
  if (!any) return;

  // Theta (chains x features) -> bf16 hi / lo, canonical K-major
  for (int idx = tid; idx < NC * TK; idx += blockDim.x) {
    const int c = idx / TK, k = idx - c * TK;
    double dv = 0.0;
    if (act_s[c] && k < Kx) dv = a.Q[(size_t)(c0 + c) * a.ldq + k];
    const __nv_bfloat16 hi = __double2bfloat16(dv);
    const __nv_bfloat16 lo = __float2bfloat16_rn((float)(dv - (double)__bfloat162float(hi)));
    const uint32_t off = kmajor_off(c, k, TK);
    *reinterpret_cast<__nv_bfloat16*>(sTh + off) = hi;
    *reinterpret_cast<__nv_bfloat16*>(sTl + off) = lo;
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, 128);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tD1 = tmem;        // columns 0..63
  const uint32_t tD2 = tmem + 64;   // columns 64..127

  const int t_begin = (int)((long long)a.n_tiles * s / a.S);
  const int t_end = (int)((long long)a.n_tiles * (s + 1) / a.S);
  const uint32_t idesc1 = make_idesc_bf16(TM, NC, 0, 0);
  const uint32_t idesc2 = make_idesc_bf16(TK, NC, 1, 1);
  const uint32_t aXh = smem_u32(sXh), aXl = smem_u32(sXl);
  const uint32_t aTh = smem_u32(sTh), aTl = smem_u32(sTl);
  const uint32_t aRh = smem_u32(sRh), aRl = smem_u32(sRl);
  uint32_t phase = 0;
  bool ok = true;
  double lp_acc = 0.0;

  for (int t = t_begin; t < t_end && ok; ++t) {
    // X tile (hi, lo): 2 x 32 KiB contiguous
    {
      const uint4* src_h = reinterpret_cast<const uint4*>(a.xt + (size_t)(2 * t) * (TM * TK));
      const uint4* src_l = reinterpret_cast<const uint4*>(a.xt + (size_t)(2 * t + 1) * (TM * TK));
      uint4* dh = reinterpret_cast<uint4*>(sXh);
      uint4* dl = reinterpret_cast<uint4*>(sXl);
      for (int i = tid; i < TILE_BYTES / 16; i += blockDim.x) {
        dh[i] = src_h[i];
        if (a.x_has_lo) dl[i] = src_l[i];
      }
    }
    fence_proxy_async();
    __syncthreads();
    // GEMM1: eta = X . Theta^T
    if (tid == 0) {
      fence_after_sync();
#pragma unroll 1
      for (int ks = 0; ks < TK / 16; ++ks) {
        const uint64_t ah = make_desc(aXh + 256 * ks, 128, (TK / 8) * 128);
        const uint64_t al = make_desc(aXl + 256 * ks, 128, (TK / 8) * 128);
        const uint64_t bh = make_desc(aTh + 256 * ks, 128, (TK / 8) * 128);
        const uint64_t bl = make_desc(aTl + 256 * ks, 128, (TK / 8) * 128);
        mma_bf16(tD1, ah, bh, idesc1, ks > 0 ? 1u : 0u);
        mma_bf16(tD1, ah, bl, idesc1, 1u);
        if (a.x_has_lo) mma_bf16(tD1, al, bh, idesc1, 1u);
      }
      mma_commit(bar);
    }
    ok = mbar_wait(bar, phase, a.err, 1);
    phase ^= 1u;
    fence_after_sync();
    // link on the eta tile: this thread's row, 64 chains
    {
      const int r = warp * 32 + lane;
      const long long row = (long long)t * TM + r;
      const bool valid = row < a.N;
      const float yv = a.yt[(size_t)t * TM + r];
      float v[64];
      tmem_ld32(tD1 + ((uint32_t)(warp * 32) << 16), v);
      tmem_ld32(tD1 + ((uint32_t)(warp * 32) << 16) + 32, v + 32);
      tmem_ld_wait();
#pragma unroll
      for (int g = 0; g < NC / 8; ++g) {
        __align__(16) __nv_bfloat16 hi8[8], lo8[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int c = g * 8 + j;
          const float eta = v[c];
          float term, resid;
          if (a.link == LINK_LOGIT) {
            const float e = __expf(-fabsf(eta));
            const float d = 1.f + e;
            const float inv = __fdividef(1.f, d);
            const float sig = eta >= 0.f ? inv : e * inv;
            term = yv * eta - (fmaxf(eta, 0.f) + __logf(d));
            resid = yv - sig;
          } else {
            const float mu = __expf(eta);
            term = yv * eta - mu;
            resid = yv - mu;
          }
          if (!valid) {
            term = 0.f;
            resid = 0.f;
          }
          v[c] = term;
          split_bf16(resid, hi8[j], lo8[j]);
        }
        const uint32_t off = (uint32_t)(g * ((TM / 8) * 128) + (r >> 3) * 128 + (r & 7) * 16);
        *reinterpret_cast<uint4*>(sRh + off) = *reinterpret_cast<const uint4*>(hi8);
        *reinterpret_cast<uint4*>(sRl + off) = *reinterpret_cast<const uint4*>(lo8);
      }
      float s0, s1;
      warp_reduce_scatter64(v, s0, s1);
      sLP[warp * NC + 2 * lane] = s0;
      sLP[warp * NC + 2 * lane + 1] = s1;
    }
    fence_before_sync();
    fence_proxy_async();
    __syncthreads();
    if (tid < NC)
      lp_acc += (double)sLP[tid] + (double)sLP[NC + tid] + (double)sLP[2 * NC + tid] +
                (double)sLP[3 * NC + tid];
    // GEMM2: G += X^T . R  (both operands MN-major)
    if (tid == 0) {
      fence_after_sync();
#pragma unroll 1
      for (int ks = 0; ks < TM / 16; ++ks) {
        const uint64_t ah = make_desc(aXh + 4096 * ks, (TM / 8) * 128 * 1, 128);
        const uint64_t al = make_desc(aXl + 4096 * ks, (TM / 8) * 128 * 1, 128);
        const uint64_t bh = make_desc(aRh + 256 * ks, 128, (TM / 8) * 128);
        const uint64_t bl = make_desc(aRl + 256 * ks, 128, (TM / 8) * 128);
        const uint32_t acc0 = (t > t_begin || ks > 0) ? 1u : 0u;
        mma_bf16(tD2, ah, bh, idesc2, acc0);
        mma_bf16(tD2, ah, bl, idesc2, 1u);
        if (a.x_has_lo) mma_bf16(tD2, al, bh, idesc2, 1u);
      }
      mma_commit(bar);
    }
    ok = mbar_wait(bar, phase, a.err, 2) && ok;
    phase ^= 1u;
    fence_after_sync();
  }
  __syncthreads();
  // gradient partials: this thread's feature row of G, 64 chains
  {
    const int k = warp * 32 + lane;
    float g[64];
    const bool have = ok && (t_end > t_begin);
    if (have) {
      tmem_ld32(tD2 + ((uint32_t)(warp * 32) << 16), g);
      tmem_ld32(tD2 + ((uint32_t)(warp * 32) << 16) + 32, g + 32);
      tmem_ld_wait();
    } else {
#pragma unroll
      for (int c = 0; c < 64; ++c) g[c] = 0.f;
    }
    int slot = -1;
    if (k < hb)
      slot = 1;
    else if (k - hb < a.K)
      slot = 4 + (k - hb);
    if (slot >= 0) {
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (act_s[c]) a.P[((size_t)s * a.C + c0 + c) * a.NP + slot] = (double)g[c];
    }
    if (tid < NC && act_s[tid]) {
      double* dst = a.P + ((size_t)s * a.C + c0 + tid) * a.NP;
      dst[0] = lp_acc;
      dst[2] = 0.0;
      dst[3] = 0.0;
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, 128);
  }
}

int tc_prepare(const ModelDesc& m, void** xtv, float** yt, int* n_tiles, cudaStream_t st) {
  __nv_bfloat16** xt = reinterpret_cast<__nv_bfloat16**>(xtv);
  const int tiles = (int)((m.N + TM - 1) / TM);
  const size_t xbytes = (size_t)tiles * 2 * TILE_BYTES;
  GBN_CUDA_TRY(cudaMalloc(xt, xbytes));
  GBN_CUDA_TRY(cudaMalloc(yt, (size_t)tiles * TM * sizeof(float)));
  const long long total = (long long)tiles * TM * TK;
  const int threads = 256;
  const int blocks = (int)std::min<long long>((total + threads - 1) / threads, 152 * 16);
  tc_prepare_tiles_kernel<<<blocks, threads, 0, st>>>(m.X, m.x_dtype, m.N, m.K, m.has_base,
                                                      tiles, *xt, m.y, *yt);
  GBN_CUDA_TRY(cudaGetLastError());
  *n_tiles = tiles;
  return GBNUTS_OK;
}

int tc_splits(const ModelDesc& m, int C) {
  const int groups = (C + NC - 1) / NC;
  int S = std::max(1, 148 / groups);
  S = std::min<long long>(S, std::max(1, m.tc_tiles));
  return S;
}

int launch_tc(const ModelDesc& m, const double* Q, int ldq, int C, const int* active,
              GradWorkspace& ws, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    GBN_CUDA_TRY(cudaFuncSetAttribute(glm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      SMEM_ALLOC));
    attr = true;
  }
  TcArgs a;
  a.xt = static_cast<const __nv_bfloat16*>(m.tc_xt);
  a.yt = m.tc_yt;
  a.N = m.N;
  a.K = m.K;
  a.has_base = m.has_base;
  a.n_tiles = m.tc_tiles;
  a.link = m.link;
  a.x_has_lo = m.x_dtype == GBNUTS_BF16 ? 0 : 1;
  a.Q = Q;
  a.ldq = ldq;
  a.C = C;
  a.active = active;
  a.P = ws.partial;
  a.NP = ws.NP;
  a.S = ws.S;
  a.err = ws.err;
  dim3 grid(ws.S, (C + NC - 1) / NC);
  glm_tc_kernel<<<grid, 128, SMEM_ALLOC, st>>>(a);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

// ------------------------------------------------------------------ probe
// One tile through both contraction layouts, for checking the descriptors:
// D1 = A . B^T (A 128x128 rows x k, B 64x128 chains x k, K-major) and
// D2 = A^T . R (R 128 rows x 64 chains; both operands MN-major).
__global__ void __launch_bounds__(128, 1)
    tc_probe_kernel(const __nv_bfloat16* A, const __nv_bfloat16* B, const __nv_bfloat16* R,
                    float* D1, float* D2, int* err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char* sX = sm + SMEM_X;
  unsigned char* sT = sm + SMEM_T;
  unsigned char* sR = sm + SMEM_R;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + SMEM_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SMEM_BAR + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < TM * TK; i += 128) {
    const int r = i / TK, k = i - r * TK;
    *reinterpret_cast<__nv_bfloat16*>(sX + kmajor_off(r, k, TK)) = A[i];
  }
  for (int i = tid; i < NC * TK; i += 128) {
    const int c = i / TK, k = i - c * TK;
    *reinterpret_cast<__nv_bfloat16*>(sT + kmajor_off(c, k, TK)) = B[i];
  }
  for (int i = tid; i < TM * NC; i += 128) {
    const int r = i / NC, c = i - r * NC;
    const uint32_t off = (uint32_t)((c >> 3) * ((TM / 8) * 128) + (r >> 3) * 128 + (r & 7) * 16 +
                                    (c & 7) * 2);
    *reinterpret_cast<__nv_bfloat16*>(sR + off) = R[i];
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, 128);
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  if (tid == 0) {
    const uint32_t idesc1 = make_idesc_bf16(TM, NC, 0, 0);
    const uint32_t idesc2 = make_idesc_bf16(TK, NC, 1, 1);
    for (int ks = 0; ks < TK / 16; ++ks)
      mma_bf16(tmem, make_desc(smem_u32(sX) + 256 * ks, 128, (TK / 8) * 128),
               make_desc(smem_u32(sT) + 256 * ks, 128, (TK / 8) * 128), idesc1, ks > 0);
    for (int ks = 0; ks < TM / 16; ++ks)
      mma_bf16(tmem + 64, make_desc(smem_u32(sX) + 4096 * ks, (TM / 8) * 128, 128),
               make_desc(smem_u32(sR) + 256 * ks, 128, (TM / 8) * 128), idesc2, ks > 0);
    mma_commit(bar);
  }
  const bool ok = mbar_wait(bar, 0, err, 3);
  fence_after_sync();
  if (ok) {
    float v[64];
    const int r = warp * 32 + lane;
    tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
    tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + 32, v + 32);
    tmem_ld_wait();
    for (int c = 0; c < 64; ++c) D1[r * 64 + c] = v[c];
    tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + 64, v);
    tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + 96, v + 32);
    tmem_ld_wait();
    for (int c = 0; c < 64; ++c) D2[r * 64 + c] = v[c];
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, 128);
  }
}

}  // namespace gbn

// Test hook (include/gbnuts_testing.h): runs the probe kernel on host arrays.
extern "C" int gbnuts_tc_probe(const uint16_t* A, const uint16_t* B, const uint16_t* R,
                               float* D1, float* D2) {
  using namespace gbn;
  void *dA, *dB, *dR, *dD1, *dD2, *dE;
  GBN_CUDA_TRY(cudaMalloc(&dA, TM * TK * 2));
  GBN_CUDA_TRY(cudaMalloc(&dB, NC * TK * 2));
  GBN_CUDA_TRY(cudaMalloc(&dR, TM * NC * 2));
  GBN_CUDA_TRY(cudaMalloc(&dD1, TM * NC * 4));
  GBN_CUDA_TRY(cudaMalloc(&dD2, TK * NC * 4));
  GBN_CUDA_TRY(cudaMalloc(&dE, 4));
  GBN_CUDA_TRY(cudaMemset(dE, 0, 4));
  GBN_CUDA_TRY(cudaMemcpy(dA, A, TM * TK * 2, cudaMemcpyHostToDevice));
  GBN_CUDA_TRY(cudaMemcpy(dB, B, NC * TK * 2, cudaMemcpyHostToDevice));
  GBN_CUDA_TRY(cudaMemcpy(dR, R, TM * NC * 2, cudaMemcpyHostToDevice));
  GBN_CUDA_TRY(cudaFuncSetAttribute(tc_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    SMEM_ALLOC));
  tc_probe_kernel<<<1, 128, SMEM_ALLOC>>>((const __nv_bfloat16*)dA, (const __nv_bfloat16*)dB,
                                          (const __nv_bfloat16*)dR, (float*)dD1, (float*)dD2,
                                          (int*)dE);
  GBN_CUDA_TRY(cudaGetLastError());
  GBN_CUDA_TRY(cudaDeviceSynchronize());
  int e = 0;
  GBN_CUDA_TRY(cudaMemcpy(&e, dE, 4, cudaMemcpyDeviceToHost));
  GBN_CUDA_TRY(cudaMemcpy(D1, dD1, TM * NC * 4, cudaMemcpyDeviceToHost));
  GBN_CUDA_TRY(cudaMemcpy(D2, dD2, TK * NC * 4, cudaMemcpyDeviceToHost));
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dR);
  cudaFree(dD1);
  cudaFree(dD2);
  cudaFree(dE);
  if (e) {
    set_last_error("tensor-core probe: wait timed out");
    return GBNUTS_SOFTWARE;
  }
  return GBNUTS_OK;
}
