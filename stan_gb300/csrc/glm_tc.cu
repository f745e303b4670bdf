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
constexpr int NUM_EPI_WARPS = 8;             // two per TMEM lane quarter (32 columns each)
constexpr int TC_THREADS = 64 + 32 * NUM_EPI_WARPS;
// pipelined kernel: two X stages (hi + lo each), Theta, R, lp scratch, barriers
constexpr int Y_BYTES = TM * 4;               // y of one tile (fp32)
constexpr int STAGE_BYTES = 2 * TILE_BYTES + 1024;  // X hi, X lo, y (padded)
constexpr int SMEM_X = 0;
constexpr int SMEM_T = SMEM_X + 2 * STAGE_BYTES;
constexpr int SMEM_R = SMEM_T + 2 * THETA_BYTES;
constexpr int SMEM_LP = SMEM_R + 2 * R_BYTES;
constexpr int SMEM_BAR = SMEM_LP + 4 * NC * 8;  // lp partials [quarter][chain]
constexpr int SMEM_TOTAL = SMEM_BAR + 256;
constexpr int SMEM_ALLOC = SMEM_TOTAL + 1024;  // slack for 1 KiB alignment
// barrier slots (uint64 each) inside SMEM_BAR
enum { B_XFULL = 0, B_XEMPTY = 2, B_D1FULL = 4, B_D1EMPTY = 6, B_RFULL = 8, B_REMPTY = 9,
       B_D2FULL = 10, B_COUNT = 11 };

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

// Warp transpose reduction: v[32] per lane (one row each) -> returns, in lane
// l, the sum over the warp's 32 rows of column l.
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
  const int lane = threadIdx.x & 31;
  float w[16];
  {
    const bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      float send = up ? v[i] : v[16 + i];
      float keep = up ? v[16 + i] : v[i];
      w[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
  }
  float x[8];
  {
    const bool up = lane & 8;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float send = up ? w[i] : w[8 + i];
      float keep = up ? w[8 + i] : w[i];
      x[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
  }
  float y[4];
  {
    const bool up = lane & 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float send = up ? x[i] : x[4 + i];
      float keep = up ? x[4 + i] : x[i];
      y[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
  }
  float z[2];
  {
    const bool up = lane & 2;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      float send = up ? y[i] : y[2 + i];
      float keep = up ? y[2 + i] : y[i];
      z[i] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
  }
  const bool up = lane & 1;
  float send = up ? z[0] : z[1], keep = up ? z[1] : z[0];
  return keep + __shfl_xor_sync(0xffffffffu, send, 1);
}

template <int LINK, bool XLO>
__global__ void __launch_bounds__(TC_THREADS, 1) glm_tc_kernel(TcArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char* sTh = sm + SMEM_T;
  unsigned char* sTl = sTh + THETA_BYTES;
  unsigned char* sRh = sm + SMEM_R;
  unsigned char* sRl = sRh + R_BYTES;
  double* sLP = reinterpret_cast<double*>(sm + SMEM_LP);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + SMEM_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SMEM_BAR + 8 * B_COUNT);
  volatile int* abort_s = reinterpret_cast<volatile int*>(sm + SMEM_BAR + 8 * B_COUNT + 8);
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
    for (int b = 0; b < 2; ++b) {
      mbar_init(&bars[B_XFULL + b], 1);
      mbar_init(&bars[B_XEMPTY + b], 1);
      mbar_init(&bars[B_D1FULL + b], 1);
      mbar_init(&bars[B_D1EMPTY + b], NUM_EPI_WARPS);
    }
    mbar_init(&bars[B_RFULL], NUM_EPI_WARPS);
    mbar_init(&bars[B_REMPTY], 1);
    mbar_init(&bars[B_D2FULL], 1);
    *abort_s = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, 256);
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tD2 = tmem + 128;

  const int t_begin = (int)((long long)a.n_tiles * s / a.S);
  const int t_end = (int)((long long)a.n_tiles * (s + 1) / a.S);
  const int n = t_end - t_begin;
  const uint32_t x_bytes = XLO ? 2u * TILE_BYTES : (uint32_t)TILE_BYTES;

  if (n > 0) {
    if (warp == 0) {
      // ---- producer: X tiles through the 2-stage ring
      if (lane == 0) {
        for (int i = 0; i < n; ++i) {
          const int b = i & 1, u = i >> 1;
          if (!mbar_wait_abortable(&bars[B_XEMPTY + b], (u & 1) ^ 1, abort_s, a.err, 11)) break;
          unsigned char* dst = sm + SMEM_X + b * STAGE_BYTES;
          const __nv_bfloat16* src = a.xt + (size_t)(2 * (t_begin + i)) * (TM * TK);
          mbar_arrive_expect_tx(&bars[B_XFULL + b], x_bytes + Y_BYTES);
          bulk_copy_g2s(dst, src, TILE_BYTES, &bars[B_XFULL + b]);
          if (XLO)
            bulk_copy_g2s(dst + TILE_BYTES, src + TM * TK, TILE_BYTES, &bars[B_XFULL + b]);
          bulk_copy_g2s(dst + 2 * TILE_BYTES, a.yt + (size_t)(t_begin + i) * TM, Y_BYTES,
                        &bars[B_XFULL + b]);
        }
      }
      __syncwarp();
    } else if (warp == 1) {
      // ---- MMA issuer: GEMM1 of tile i, then GEMM2 of tile i-1
      if (lane == 0) {
        const uint32_t idesc1 = make_idesc_bf16(TM, NC, 0, 0);
        const uint32_t idesc2 = make_idesc_bf16(TK, NC, 1, 1);
        const uint32_t aTh = smem_u32(sTh), aTl = smem_u32(sTl);
        const uint32_t aRh = smem_u32(sRh), aRl = smem_u32(sRl);
        bool ok = true;
        auto gemm2 = [&](int j) -> bool {
          if (!mbar_wait_abortable(&bars[B_RFULL], j & 1, abort_s, a.err, 13)) return false;
          fence_after_sync();
          const uint32_t aXh = smem_u32(sm + SMEM_X + (j & 1) * STAGE_BYTES);
          const uint32_t aXl = aXh + TILE_BYTES;
#pragma unroll 1
          for (int ks = 0; ks < TM / 16; ++ks) {
            const uint64_t ah = make_desc(aXh + 4096 * ks, (TM / 8) * 128, 128);
            const uint64_t al = make_desc(aXl + 4096 * ks, (TM / 8) * 128, 128);
            const uint64_t bh = make_desc(aRh + 256 * ks, 128, (TM / 8) * 128);
            const uint64_t bl = make_desc(aRl + 256 * ks, 128, (TM / 8) * 128);
            const uint32_t acc0 = (j > 0 || ks > 0) ? 1u : 0u;
            mma_bf16(tD2, ah, bh, idesc2, acc0);
            mma_bf16(tD2, ah, bl, idesc2, 1u);
            if (XLO) mma_bf16(tD2, al, bh, idesc2, 1u);
          }
          mma_commit(&bars[B_REMPTY]);
          mma_commit(&bars[B_XEMPTY + (j & 1)]);
          return true;
        };
        for (int i = 0; i < n && ok; ++i) {
          const int b = i & 1, u = i >> 1;
          ok = mbar_wait_abortable(&bars[B_XFULL + b], u & 1, abort_s, a.err, 12) &&
               mbar_wait_abortable(&bars[B_D1EMPTY + b], (u & 1) ^ 1, abort_s, a.err, 14);
          if (!ok) break;
          fence_after_sync();
          const uint32_t aXh = smem_u32(sm + SMEM_X + b * STAGE_BYTES);
          const uint32_t aXl = aXh + TILE_BYTES;
          const uint32_t tD1 = tmem + 64 * b;
#pragma unroll 1
          for (int ks = 0; ks < TK / 16; ++ks) {
            const uint64_t ah = make_desc(aXh + 256 * ks, 128, (TK / 8) * 128);
            const uint64_t al = make_desc(aXl + 256 * ks, 128, (TK / 8) * 128);
            const uint64_t bh = make_desc(aTh + 256 * ks, 128, (TK / 8) * 128);
            const uint64_t bl = make_desc(aTl + 256 * ks, 128, (TK / 8) * 128);
            mma_bf16(tD1, ah, bh, idesc1, ks > 0 ? 1u : 0u);
            mma_bf16(tD1, ah, bl, idesc1, 1u);
            if (XLO) mma_bf16(tD1, al, bh, idesc1, 1u);
          }
          mma_commit(&bars[B_D1FULL + b]);
          if (i > 0) ok = gemm2(i - 1);
        }
        if (ok) ok = gemm2(n - 1);
        mma_commit(&bars[B_D2FULL]);
      }
      __syncwarp();
    } else {
      // ---- epilogue: link on eta, R to shared memory, lp partial sums.
      // Warp w (2..9): TMEM lane quarter q = w % 4 (rows 32q..32q+31),
      // chain half h (columns 32h..32h+31).
      const int q = warp & 3;
      const int h = (warp - 2) >> 2;
      const int r = q * 32 + lane;
      double lp_acc = 0.0;
      bool ok = true;
      for (int i = 0; i < n && ok; ++i) {
        const int b = i & 1, u = i >> 1;
        const int t = t_begin + i;
        if (!warp_wait(&bars[B_D1FULL + b], u & 1, abort_s, a.err, 15)) {
          ok = false;
          break;
        }
        fence_after_sync();
        float v[32];
        tmem_ld32(tmem + 64 * b + 32 * h + ((uint32_t)(q * 32) << 16), v);
        tmem_ld_wait();
        fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_D1EMPTY + b]);
        const long long row = (long long)t * TM + r;
        const bool valid = row < a.N;
        const float yv =
            reinterpret_cast<const float*>(sm + SMEM_X + b * STAGE_BYTES + 2 * TILE_BYTES)[r];
        uint32_t rh[16], rl[16];
#pragma unroll
        for (int c = 0; c < 32; c += 2) {
          float res[2];
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const float eta = v[c + j];
            float term, resid;
            if (LINK == LINK_LOGIT) {
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
            v[c + j] = valid ? term : 0.f;
            res[j] = valid ? resid : 0.f;
          }
          const __nv_bfloat162 hp = __floats2bfloat162_rn(res[0], res[1]);
          const float2 hf = __bfloat1622float2(hp);
          const __nv_bfloat162 lp2 = __floats2bfloat162_rn(res[0] - hf.x, res[1] - hf.y);
          rh[c >> 1] = *reinterpret_cast<const uint32_t*>(&hp);
          rl[c >> 1] = *reinterpret_cast<const uint32_t*>(&lp2);
        }
        if (!warp_wait(&bars[B_REMPTY], (i & 1) ^ 1, abort_s, a.err, 16)) {
          ok = false;
          break;
        }
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          const int cg = 4 * h + g;  // chain group of 8
          const uint32_t off = (uint32_t)(cg * ((TM / 8) * 128) + (r >> 3) * 128 + (r & 7) * 16);
          *reinterpret_cast<uint4*>(sRh + off) =
              make_uint4(rh[4 * g], rh[4 * g + 1], rh[4 * g + 2], rh[4 * g + 3]);
          *reinterpret_cast<uint4*>(sRl + off) =
              make_uint4(rl[4 * g], rl[4 * g + 1], rl[4 * g + 2], rl[4 * g + 3]);
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_RFULL]);
        lp_acc += (double)warp_reduce_scatter32(v);
      }
      sLP[q * NC + 32 * h + lane] = lp_acc;
      // gradient partials: this thread's feature row of G, 32 chains
      if (ok && warp_wait(&bars[B_D2FULL], 0, abort_s, a.err, 17)) {
        fence_after_sync();
        float g[32];
        tmem_ld32(tD2 + 32 * h + ((uint32_t)(q * 32) << 16), g);
        tmem_ld_wait();
        const int k = q * 32 + lane;
        int slot = -1;
        if (k < hb)
          slot = 1;
        else if (k - hb < a.K)
          slot = 4 + (k - hb);
        if (slot >= 0) {
#pragma unroll
          for (int c = 0; c < 32; ++c)
            if (act_s[32 * h + c])
              a.P[((size_t)s * a.C + c0 + 32 * h + c) * a.NP + slot] = (double)g[c];
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid < NC && act_s[tid]) {
    double* dst = a.P + ((size_t)s * a.C + c0 + tid) * a.NP;
    double lp = 0.0;
    if (n > 0) lp = sLP[tid] + sLP[NC + tid] + sLP[2 * NC + tid] + sLP[3 * NC + tid];
    dst[0] = lp;
    dst[2] = 0.0;
    dst[3] = 0.0;
    if (n == 0) {
      for (int k = 0; k < Kx; ++k) dst[k < hb ? 1 : 4 + (k - hb)] = 0.0;
    }
  }
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, 256);
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
    GBN_CUDA_TRY(cudaFuncSetAttribute(glm_tc_kernel<LINK_LOGIT, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_ALLOC));
    GBN_CUDA_TRY(cudaFuncSetAttribute(glm_tc_kernel<LINK_LOGIT, false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_ALLOC));
    GBN_CUDA_TRY(cudaFuncSetAttribute(glm_tc_kernel<LINK_POISSON_LOG, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_ALLOC));
    GBN_CUDA_TRY(cudaFuncSetAttribute(glm_tc_kernel<LINK_POISSON_LOG, false>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_ALLOC));
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
  if (m.link == LINK_LOGIT) {
    if (a.x_has_lo)
      glm_tc_kernel<LINK_LOGIT, true><<<grid, TC_THREADS, SMEM_ALLOC, st>>>(a);
    else
      glm_tc_kernel<LINK_LOGIT, false><<<grid, TC_THREADS, SMEM_ALLOC, st>>>(a);
  } else {
    if (a.x_has_lo)
      glm_tc_kernel<LINK_POISSON_LOG, true><<<grid, TC_THREADS, SMEM_ALLOC, st>>>(a);
    else
      glm_tc_kernel<LINK_POISSON_LOG, false><<<grid, TC_THREADS, SMEM_ALLOC, st>>>(a);
  }
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
