// Batched GLM log density and gradient for wide designs (K + intercept > 128)
// on the tcgen05 tensor cores (precisions GBNUTS_PREC_BF16X3 and
// GBNUTS_PREC_BF16, logistic and Poisson), chains on the MMA's N dimension.
//
// A CTA owns NC = 32 chains and a range of 128-row tiles of X, with every
// feature: the chains' coefficients Theta^T (bf16 hi / lo, 32 chains x up to
// 512 features, 64 KiB) stay in shared memory as the B operand, so no
// partial sums cross CTAs.  X is stored per (tile, 128-feature slab) as one
// 128 x 128 bf16 block (the canonical K-major core-matrix layout) and
// streams through a 4-stage ring of slab blocks, each tile twice:
//
//   GEMM1  eta^T (128 rows x 32 chains) = sum_f X_tile,f . Theta_f^T   (A = X,
//          K-major; accumulates over the F slabs into TMEM, two buffers)
//   link   one epilogue thread per row: lp terms of its 32 chains (summed over
//          the warp's rows by a transpose-reduce), residual r = dlp/deta as
//          bf16 hi / lo into R^T (128 rows x 32 chains, shared memory, two
//          buffers)
//   GEMM2  G_f^T (128 features x 32 chains) += X_tile,f^T . R^T   (A = the
//          same X block read MN-major; one TMEM accumulator per slab)
//
// In the split form the hi and lo parts ride on one MMA each way: B is
// [Theta_hi^T | Theta_lo^T] (64 columns) in GEMM1 and [R_hi^T | R_lo^T] in
// GEMM2, so each X slice is read once per k-step (the MMAs of this shape are
// bound by their shared-memory operand reads); the two 32-column halves of
// eta and of G are added in the epilogue.
//
// The MMA thread interleaves GEMM1 of tile i + 1 with GEMM2 of tile i, so the
// link of a tile overlaps the next tile's GEMM1; the producer loads the slab
// blocks in the order the MMAs read them.  X stored in bf16 is exact; X stored
// in fp32 or fp64 is split into bf16 hi and lo parts laid out as 2 (K +
// intercept) features [hi | lo] with Theta repeated over both halves, and the
// gradient of feature k is the sum of its hi and lo columns (two split
// partials).  Theta carries log2(e), so eta comes out in base-2 units for the
// MUFU ex2 / lg2, as in the narrow kernel (glm_tct.cu).  Every wait is bounded.
//
// TMEM (512 columns): eta buffers [0, 64) and [64, 128), G_f [128 + 64 f, ...)
// (64 columns each: the hi product, then the lo product; 32 used without the
// split).
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"
#include "tc_common.cuh"

namespace gbn {
using namespace tc;

namespace wide {

constexpr int TM = 128;                 // rows per tile
constexpr int TF = 128;                 // features per slab
constexpr int F = 4;                    // slabs; narrower designs pad
constexpr int NC = 32;                  // chains per CTA (MMA N)
constexpr int SLAB_BYTES = TM * TF * 2;
constexpr int STAGES = 4;
constexpr int TH_PART = NC * TF * 2;    // one slab's Theta^T, one bf16 part (8 KiB)
constexpr int R_PART = TM * NC * 2;     // one residual part (8 KiB); a buffer holds two
constexpr int NUM_EPI_WARPS = 4;
constexpr int THREADS = 64 + 32 * NUM_EPI_WARPS;
constexpr int SMEM_X = 0;
constexpr int SMEM_TH = SMEM_X + STAGES * SLAB_BYTES;    // [F][hi, lo] 8 KiB blocks
constexpr int SMEM_R = SMEM_TH + F * 2 * TH_PART;        // [2 buffers][hi, lo]
constexpr int SMEM_Y = SMEM_R + 2 * 2 * R_PART;          // [2][TM] fp32
constexpr int SMEM_LP = SMEM_Y + 2 * TM * 4;             // [4 quarters][NC] doubles
constexpr int SMEM_BAR = SMEM_LP + 4 * NC * 8;
constexpr int SMEM_TOTAL = SMEM_BAR + 256;
constexpr int SMEM_ALLOC = SMEM_TOTAL + 128;             // slack for 128-byte alignment
static_assert(SMEM_ALLOC + 4 * NC <= 227 * 1024, "shared memory of one CTA");
constexpr uint32_t COL_D1 = 0, COL_G = 128;
constexpr int TMEM_COLS = 512;
constexpr float kLn2f = 0.69314718f;

enum {
  B_XFULL = 0, B_XEMPTY = STAGES, B_YFULL = 2 * STAGES, B_YEMPTY = B_YFULL + 2,
  B_D1FULL = B_YEMPTY + 2, B_D1EMPTY = B_D1FULL + 2, B_RFULL = B_D1EMPTY + 2,
  B_REMPTY = B_RFULL + 2, B_THETA = B_REMPTY + 2, B_D2FULL = B_THETA + 1,
  B_COUNT = B_D2FULL + 1
};

// GEMM1 A: the 128 rows of a slab block, K-major, features 16 ks ..
__device__ __forceinline__ uint64_t desc_x_rows(uint32_t blk, int ks) {
  return make_desc(blk + 256 * ks, 128, (TF / 8) * 128);
}
// GEMM2 A: the same block MN-major (features x rows), rows 16 ks ..
__device__ __forceinline__ uint64_t desc_x_feats(uint32_t blk, int ks) {
  return make_desc(blk + 4096 * ks, (TF / 8) * 128, 128);
}
// GEMM1 B: Theta^T of one slab (32 chains x 128 features), K-major
__device__ __forceinline__ uint64_t desc_theta(uint32_t part, int ks) {
  return make_desc(part + 256 * ks, 128, (TF / 8) * 128);
}
// GEMM2 B: R^T (rows x 64 columns: the 32 chains' hi parts, then their lo
// parts) MN-major, columns contiguous: element (row r, column c) at
// (r / 8) 1024 + (c / 8) 128 + (r % 8) 16 + (c % 8) 2
__device__ __forceinline__ uint32_t r_off(int r, int c) {
  return (uint32_t)((r >> 3) * (2 * NC / 8) * 128 + (c >> 3) * 128 + (r & 7) * 16 + (c & 7) * 2);
}
__device__ __forceinline__ uint64_t desc_r(uint32_t buf, int ks) {
  return make_desc(buf + 2 * (2 * NC / 8) * 128 * ks, (2 * NC / 8) * 128, 128);
}

__device__ __forceinline__ void two_sum_add(float2& s, float v) {
  const float t = s.x + v;
  const float bp = t - s.x;
  const float err = (s.x - (t - bp)) + (v - bp);
  s.x = t;
  s.y += err;
}

}  // namespace wide

struct WideArgs {
  const uint16_t* xt;  // [tile][slab] 128 x 128 bf16 blocks
  const float* yt;     // y per tile row
  long long N;
  int kx;              // K + intercept
  int doubled;         // features are [X hi | X lo] (2 kx of them)
  int has_base;
  int n_tiles;
  const double* Q;
  int ldq, C;
  const int* active;
  double* P;
  int NP, S;  // S: row splits (the partials hold S, or 2 S when doubled, split rows)
  int* err;
};

template <int LINK, bool SPLIT>
__global__ void __launch_bounds__(wide::THREADS, 1) glm_wide_kernel(WideArgs a) {
  using namespace wide;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + SMEM_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SMEM_BAR + 8 * B_COUNT);
  volatile int* abort_s = reinterpret_cast<volatile int*>(sm + SMEM_BAR + 8 * B_COUNT + 8);
  double* sLP = reinterpret_cast<double*>(sm + SMEM_LP);
  __shared__ int act_s[NC];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s = blockIdx.x;
  const int c0 = blockIdx.y * NC;
  if (tid < NC) {
    const int cg = c0 + tid;
    act_s[tid] = (cg < a.C) && (a.active == nullptr || a.active[cg] != 0);
  }
  const int any = __syncthreads_or(tid < NC ? act_s[tid] : 0);
  if (!any) return;

  if (tid == 0) {
    for (int b = 0; b < STAGES; ++b) {
      mbar_init(&bars[B_XFULL + b], 1);
      mbar_init(&bars[B_XEMPTY + b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&bars[B_YFULL + b], 1);
      mbar_init(&bars[B_YEMPTY + b], NUM_EPI_WARPS);
      mbar_init(&bars[B_D1FULL + b], 1);
      mbar_init(&bars[B_D1EMPTY + b], NUM_EPI_WARPS);
      mbar_init(&bars[B_RFULL + b], NUM_EPI_WARPS);
      mbar_init(&bars[B_REMPTY + b], 1);
    }
    mbar_init(&bars[B_THETA], NUM_EPI_WARPS);
    mbar_init(&bars[B_D2FULL], 1);
    *abort_s = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, TMEM_COLS);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  const int t_begin = (int)((long long)a.n_tiles * s / a.S);
  const int t_end = (int)((long long)a.n_tiles * (s + 1) / a.S);
  const int n = t_end - t_begin;
  const uint32_t sm_base = smem_u32(sm);
  // Passes over the slab blocks, in the order the MMAs read them: GEMM1 of
  // tile 0, then for i >= 1 GEMM1 of tile i and GEMM2 of tile i - 1, then
  // GEMM2 of tile n - 1.  Pass p: tile pass_tile(p), GEMM2 iff pass_g2(p).
  const int n_pass = 2 * n;

  if (n > 0) {
    if (warp == 0) {
      // ---- producer
      if (lane == 0) {
        int j = 0;  // slab block loads so far
        bool ok = true;
        for (int p = 0; p < n_pass && ok; ++p) {
          // p = 0: G1(0); p odd: G1((p + 1) / 2) for p < 2n - 1; p even >= 2: G2(p / 2 - 1);
          // the last pass (p = 2n - 1) is G2(n - 1)
          bool g2;
          int t;
          if (p == 0) {
            g2 = false;
            t = 0;
          } else if (p == n_pass - 1) {
            g2 = true;
            t = n - 1;
          } else if (p & 1) {
            g2 = false;
            t = (p + 1) / 2;
          } else {
            g2 = true;
            t = p / 2 - 1;
          }
          if (!g2) {
            const int yb = t & 1;
            ok = mbar_wait_abortable(&bars[B_YEMPTY + yb], ((t >> 1) & 1) ^ 1, abort_s, a.err, 60);
            if (!ok) break;
            mbar_arrive_expect_tx(&bars[B_YFULL + yb], TM * 4);
            bulk_copy_g2s(sm + SMEM_Y + yb * TM * 4, a.yt + (size_t)(t_begin + t) * TM, TM * 4,
                          &bars[B_YFULL + yb]);
          }
          for (int f = 0; f < F; ++f, ++j) {
            const int st = j % STAGES, u = j / STAGES;
            ok = mbar_wait_abortable(&bars[B_XEMPTY + st], (u & 1) ^ 1, abort_s, a.err, 61);
            if (!ok) break;
            mbar_arrive_expect_tx(&bars[B_XFULL + st], SLAB_BYTES);
            bulk_copy_g2s(sm + SMEM_X + st * SLAB_BYTES,
                          a.xt + ((size_t)(t_begin + t) * F + f) * (TM * TF), SLAB_BYTES,
                          &bars[B_XFULL + st]);
          }
        }
      }
      __syncwarp();
    } else if (warp == 1) {
      // ---- MMA issuer
      if (lane == 0) {
        constexpr int NB = SPLIT ? 2 * NC : NC;  // B columns: hi (and lo) parts
        const uint32_t id1 = make_idesc_bf16(TM, NB, 0, 0);
        const uint32_t id2 = make_idesc_bf16(TF, NB, 1, 1);
        bool ok = mbar_wait_abortable(&bars[B_THETA], 0, abort_s, a.err, 62);
        fence_after_sync();
        int j = 0;
        for (int p = 0; p < n_pass && ok; ++p) {
          bool g2;
          int t;
          if (p == 0) {
            g2 = false;
            t = 0;
          } else if (p == n_pass - 1) {
            g2 = true;
            t = n - 1;
          } else if (p & 1) {
            g2 = false;
            t = (p + 1) / 2;
          } else {
            g2 = true;
            t = p / 2 - 1;
          }
          const int b = t & 1;
          if (!g2) {
            // eta buffer b free: the epilogue has read tile t - 2's eta
            ok = mbar_wait_abortable(&bars[B_D1EMPTY + b], ((t >> 1) & 1) ^ 1, abort_s, a.err, 63);
          } else {
            ok = mbar_wait_abortable(&bars[B_RFULL + b], (t >> 1) & 1, abort_s, a.err, 64);
          }
          if (!ok) break;
          fence_after_sync();
          for (int f = 0; f < F; ++f, ++j) {
            const int st = j % STAGES;
            ok = mbar_wait_abortable(&bars[B_XFULL + st], (j / STAGES) & 1, abort_s, a.err, 65);
            if (!ok) break;
            fence_after_sync();
            const uint32_t xb = sm_base + SMEM_X + st * SLAB_BYTES;
            if (!g2) {
              // B: this slab's [Theta_hi^T | Theta_lo^T], 64 rows K-major
              // (the lo block follows the hi block)
              const uint32_t d1 = tmem + COL_D1 + 64 * b;
              const uint32_t th = sm_base + SMEM_TH + f * 2 * TH_PART;
#pragma unroll 4
              for (int ks = 0; ks < TF / 16; ++ks)
                mma_bf16(d1, desc_x_rows(xb, ks), desc_theta(th, ks), id1,
                         (f > 0 || ks > 0) ? 1u : 0u);
            } else {
              const uint32_t g = tmem + COL_G + 64 * f;
              const uint32_t rb = sm_base + SMEM_R + b * 2 * R_PART;
#pragma unroll 4
              for (int ks = 0; ks < TM / 16; ++ks)
                mma_bf16(g, desc_x_feats(xb, ks), desc_r(rb, ks), id2, (t > 0 || ks > 0) ? 1u : 0u);
            }
            mma_commit(&bars[B_XEMPTY + st]);
          }
          if (!ok) break;
          mma_commit(g2 ? &bars[B_REMPTY + b] : &bars[B_D1FULL + b]);
        }
        mma_commit(&bars[B_D2FULL]);
        // no MMA may still run when tensor memory is released
        mbar_wait(&bars[B_D2FULL], 0, a.err, 69);
      }
      __syncwarp();
    } else {
      // ---- epilogue: warp w owns TMEM lane quarter q = w % 4: tile rows
      // 32 q .. 32 q + 31 (GEMM1) and slab features 32 q .. (GEMM2)
      const int q = warp & 3;
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
      {
        // log2(e) Theta^T into shared memory: thread e writes chain e % 32,
        // feature pairs e / 32, e / 32 + 4, ...
        const int e = tid - 64;
        const int c = e & 31;
        const bool act = act_s[c] != 0;
        const double* th = a.Q + (size_t)(act ? c0 + c : 0) * a.ldq;
        for (int jp = e >> 5; jp < F * TF / 2; jp += NUM_EPI_WARPS) {
          double d2[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int fj = 2 * jp + h;
            const int k = fj < a.kx ? fj : (a.doubled && fj < 2 * a.kx ? fj - a.kx : -1);
            d2[h] = (act && k >= 0) ? th[k] : 0.0;
          }
          uint32_t wh, wl;
          theta_words(d2[0], d2[1], wh, wl);
          const int f = (2 * jp) / TF, kk = (2 * jp) % TF;
          const uint32_t off = kmajor_off(c, kk, TF);
          *reinterpret_cast<uint32_t*>(sm + SMEM_TH + f * 2 * TH_PART + off) = wh;
          *reinterpret_cast<uint32_t*>(sm + SMEM_TH + f * 2 * TH_PART + TH_PART + off) = wl;
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_THETA]);
      }
      const int r = 32 * q + lane;  // tile row of this thread
      float2 acc = make_float2(0.f, 0.f);  // lp of chain `lane` over this warp's rows
      bool ok = true;
      for (int t = 0; t < n && ok; ++t) {
        const int b = t & 1;
        const uint32_t par = (t >> 1) & 1;
        if (!warp_wait(&bars[B_D1FULL + b], par, abort_s, a.err, 66) ||
            !warp_wait(&bars[B_YFULL + b], par, abort_s, a.err, 67)) {
          ok = false;
          break;
        }
        fence_after_sync();
        float v[NC];
        tmem_ld32(lane_addr + COL_D1 + 64 * b, v);
        if (SPLIT) {
          float vl[NC];
          tmem_ld32(lane_addr + COL_D1 + 64 * b + NC, vl);
          tmem_ld_wait();
#pragma unroll
          for (int c = 0; c < NC; ++c) v[c] += vl[c];
        }
        tmem_ld_wait();
        const float yv = reinterpret_cast<const float*>(sm + SMEM_Y + b * TM * 4)[r];
        fence_before_sync();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&bars[B_D1EMPTY + b]);
          mbar_arrive(&bars[B_YEMPTY + b]);
        }
        const bool valid = (long long)(t_begin + t) * TM + r < a.N;
        float lt[NC];
        uint32_t wh[NC / 2], wl[NC / 2];
#pragma unroll
        for (int c = 0; c < NC; c += 2) {
          float res[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float x = v[c + h];
            float term, rr;
            if (LINK == LINK_LOGIT) {
              const float ex = ex2_approx(-fabsf(x));
              const float dd = 1.f + ex;
              const float inv = rcp_approx(dd);
              const float sig = x >= 0.f ? inv : ex * inv;
              term = kLn2f * (yv * x - fmaxf(x, 0.f) - lg2_approx(dd));
              rr = yv - sig;
            } else {
              const float mu = ex2_approx(x);
              term = kLn2f * (yv * x) - mu;
              rr = yv - mu;
            }
            if (!valid) {
              term = 0.f;
              rr = 0.f;
            }
            lt[c + h] = term;
            res[h] = rr;
          }
          const __nv_bfloat162 hp = __floats2bfloat162_rn(res[0], res[1]);
          const float2 hf = __bfloat1622float2(hp);
          const __nv_bfloat162 lo = __floats2bfloat162_rn(res[0] - hf.x, res[1] - hf.y);
          wh[c >> 1] = *reinterpret_cast<const uint32_t*>(&hp);
          wl[c >> 1] = *reinterpret_cast<const uint32_t*>(&lo);
        }
        // sum over the warp's 32 rows, chain by chain: a transpose-reduce
        // leaves chain `lane`'s sum in lane `lane` (fixed order)
#pragma unroll
        for (int w = 16; w >= 1; w >>= 1) {
          const bool up = (lane & w) != 0;
#pragma unroll
          for (int k = 0; k < w; ++k) {
            const float send = up ? lt[k] : lt[k + w];
            const float recv = __shfl_xor_sync(0xffffffffu, send, w);
            lt[k] = (up ? lt[k + w] : lt[k]) + recv;
          }
        }
        two_sum_add(acc, lt[0]);
        // residual buffer b free: GEMM2 of tile t - 2 is done
        if (!warp_wait(&bars[B_REMPTY + b], par ^ 1, abort_s, a.err, 68)) {
          ok = false;
          break;
        }
        unsigned char* rbuf = sm + SMEM_R + b * 2 * R_PART;
#pragma unroll
        for (int cg = 0; cg < NC / 8; ++cg) {
          *reinterpret_cast<uint4*>(rbuf + r_off(r, 8 * cg)) =
              make_uint4(wh[4 * cg], wh[4 * cg + 1], wh[4 * cg + 2], wh[4 * cg + 3]);
          if (SPLIT)
            *reinterpret_cast<uint4*>(rbuf + r_off(r, NC + 8 * cg)) =
                make_uint4(wl[4 * cg], wl[4 * cg + 1], wl[4 * cg + 2], wl[4 * cg + 3]);
        }
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_RFULL + b]);
      }
      sLP[q * NC + lane] = (double)acc.x + (double)acc.y;
      // gradient partials: slab f's features 32 q + lane, all 32 chains
      if (ok && warp_wait(&bars[B_D2FULL], 0, abort_s, a.err, 70)) {
        fence_after_sync();
        for (int f = 0; f < F; ++f) {
          float g[NC];
          tmem_ld32(lane_addr + COL_G + 64 * f, g);
          if (SPLIT) {
            float gl[NC];
            tmem_ld32(lane_addr + COL_G + 64 * f + NC, gl);
            tmem_ld_wait();
#pragma unroll
            for (int c = 0; c < NC; ++c) g[c] += gl[c];
          }
          tmem_ld_wait();
          const int fj = f * TF + 32 * q + lane;
          int k = fj, part = 0;
          if (fj >= a.kx) {
            if (!a.doubled || fj >= 2 * a.kx) continue;
            k = fj - a.kx;
            part = 1;
          }
          const int col = k < a.has_base ? 1 : 4 + (k - a.has_base);
          for (int c = 0; c < NC; ++c) {
            if (!act_s[c]) continue;
            a.P[((size_t)(part * a.S + s) * a.C + c0 + c) * a.NP + col] = (double)g[c];
          }
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid < NC && act_s[tid]) {
    double* dst = a.P + ((size_t)s * a.C + c0 + tid) * a.NP;
    double lp = 0.0;
    if (n > 0)
      for (int k = 0; k < 4; ++k) lp += sLP[k * NC + tid];
    dst[0] = lp;
    dst[2] = 0.0;
    dst[3] = 0.0;
    if (n == 0)
      for (int k = 0; k < a.kx; ++k) dst[k < a.has_base ? 1 : 4 + (k - a.has_base)] = 0.0;
    if (a.doubled) {
      double* d2 = a.P + ((size_t)(a.S + s) * a.C + c0 + tid) * a.NP;
      d2[0] = 0.0;
      d2[2] = 0.0;
      d2[3] = 0.0;
      if (n == 0)
        for (int k = 0; k < a.kx; ++k) d2[k < a.has_base ? 1 : 4 + (k - a.has_base)] = 0.0;
    }
  }
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ------------------------------------------------------------------ host side

int wide_slabs(const ModelDesc& m) {
  const int kx = m.K + m.has_base;
  const int kf = m.x_dtype == GBNUTS_BF16 ? kx : 2 * kx;
  if (kf <= wide::TF) return 0;           // the narrow kernel's range
  if (kf <= wide::F * wide::TF) return wide::F;  // narrower designs pad to F slabs
  return 0;
}

// X (any storage type) -> [tile][slab] 128 x 128 bf16 blocks, K-major core
// matrices; features [X | 1 intercept first] or, when doubled, [hi | lo].
__global__ void wide_tiles_kernel(const void* X, int x_dtype, long long N, int K, int has_base,
                                  int kx, int doubled, int F, int n_tiles, uint16_t* xt) {
  using namespace wide;
  const long long total = (long long)n_tiles * F * TM * TF;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long blk = i / (TM * TF);
    const int e = (int)(i - blk * (TM * TF));
    const long long t = blk / F;
    const int f = (int)(blk - t * F);
    const int r = e / TF, kk = e - r * TF;
    const long long row = t * TM + r;
    const int fj = f * TF + kk;
    int k = fj, part = 0;
    if (fj >= kx) {
      k = (doubled && fj < 2 * kx) ? fj - kx : -1;
      part = 1;
    }
    float v = 0.f;
    if (row < N && k >= 0) {
      if (k < has_base) {
        v = 1.f;
      } else {
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
    const uint16_t bits = __bfloat16_as_ushort(part ? lo : hi);
    xt[blk * (TM * TF) + kmajor_off(r, kk, TF) / 2] = bits;
  }
}

__global__ void wide_y_kernel(long long N, int n_tiles, const double* y, float* yt) {
  const long long total = (long long)n_tiles * wide::TM;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x)
    yt[i] = i < N ? (float)y[i] : 0.f;
}

int wide_prepare(const ModelDesc& m, void** xt, float** yt, int* n_tiles, cudaStream_t st) {
  using namespace wide;
  const int F = wide_slabs(m);
  if (F == 0) {
    set_last_error("the wide tensor-core form takes K + intercept up to 512 (X in bf16) or "
                   "256 (X in fp32 / fp64)");
    return GBNUTS_USAGE;
  }
  const int tiles = (int)((m.N + TM - 1) / TM);
  const int kx = m.K + m.has_base;
  const int doubled = m.x_dtype != GBNUTS_BF16;
  GBN_CUDA_TRY(cudaMalloc(xt, (size_t)tiles * F * SLAB_BYTES));
  const int grid = device_sm_count() * 16;
  const long long total = (long long)tiles * F * TM * TF;
  wide_tiles_kernel<<<(int)std::min<long long>((total + 255) / 256, grid), 256, 0, st>>>(
      m.X, m.x_dtype, m.N, m.K, m.has_base, kx, doubled, F, tiles, static_cast<uint16_t*>(*xt));
  GBN_CUDA_TRY(cudaGetLastError());
  if (*yt == nullptr) {
    GBN_CUDA_TRY(cudaMalloc(yt, (size_t)tiles * TM * sizeof(float)));
    wide_y_kernel<<<std::max(1, std::min(grid, (tiles * TM + 255) / 256)), 256, 0, st>>>(
        m.N, tiles, m.y, *yt);
    GBN_CUDA_TRY(cudaGetLastError());
  }
  *n_tiles = tiles;
  return GBNUTS_OK;
}

int wide_splits(const ModelDesc& m, int C) {
  const int F = wide_slabs(m);
  if (F == 0) return 1;
  const int blocks = (C + wide::NC - 1) / wide::NC;
  const int tiles = (int)((m.N + wide::TM - 1) / wide::TM);
  int S = std::max(1, device_sm_count() / blocks);
  S = std::min(S, std::max(1, tiles));
  return S;
}

template <int LINK, bool SPLIT>
static int launch_wide_t(const WideArgs& a, int blocks, cudaStream_t st) {
  using namespace wide;
  int rc = ensure_smem(glm_wide_kernel<LINK, SPLIT>, SMEM_ALLOC);
  if (rc) return rc;
  glm_wide_kernel<LINK, SPLIT><<<dim3(a.S, blocks), THREADS, SMEM_ALLOC, st>>>(a);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

int launch_wide(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
                const int* active, GradWorkspace& ws, cudaStream_t st) {
  const int F = wide_slabs(m);
  if (F == 0 || m.wide_xt == nullptr || m.tc_yt == nullptr) {
    set_last_error("the wide tensor-core form is not prepared for this model");
    return GBNUTS_SOFTWARE;
  }
  const bool doubled = m.x_dtype != GBNUTS_BF16;
  WideArgs a;
  a.xt = static_cast<const uint16_t*>(m.wide_xt);
  a.yt = m.tc_yt;
  a.N = m.N;
  a.kx = m.K + m.has_base;
  a.doubled = doubled ? 1 : 0;
  a.has_base = m.has_base;
  a.n_tiles = m.wide_tiles;
  a.Q = Q;
  a.ldq = ldq;
  a.C = C;
  a.active = active;
  a.P = ws.partial;
  a.NP = ws.NP;
  a.S = doubled ? ws.S / 2 : ws.S;
  a.err = ws.err;
  const int blocks = (C + wide::NC - 1) / wide::NC;
  const bool split = precision == GBNUTS_PREC_BF16X3;
  if (m.link == LINK_LOGIT)
    return split ? launch_wide_t<LINK_LOGIT, true>(a, blocks, st)
                 : launch_wide_t<LINK_LOGIT, false>(a, blocks, st);
  return split ? launch_wide_t<LINK_POISSON_LOG, true>(a, blocks, st)
               : launch_wide_t<LINK_POISSON_LOG, false>(a, blocks, st);
}

}  // namespace gbn

