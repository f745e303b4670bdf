// Batched GLM log density and gradient on the tcgen05 tensor cores, chains on
// the M dimension (precisions GBNUTS_PREC_BF16X3 and GBNUTS_PREC_BF16 for the
// logistic and Poisson GLMs, GBNUTS_PREC_F16X3 for the logistic GLM).
//
// A CTA owns 128 chains (one per TMEM lane) and a range of 128-row tiles of X,
// one tile per pass:
//   GEMM1  eta^T (128 chains x 128 rows)  = Theta . X_tile^T     A = Theta in TMEM
//   link   term, r = d lp / d eta         per (chain, row), fp32, read from TMEM
//   GEMM2  G^T (128 chains x NF feats)   += R . X_tile           A = R in TMEM
// Theta and R are A operands held in tensor memory (bf16 hi and lo parts,
// two elements per 32-bit column), so every MMA reads only its X operand
// from shared memory: GEMM1 reads X K-major (rows x features) and GEMM2 the
// same bytes MN-major (features x rows).  An MMA instruction costs about the
// same time for any N up to 128, so GEMM1 takes a whole 128-row tile as N,
// and contraction steps past the last feature are skipped.  X, Theta and R
// are each split into bf16 hi + lo and the three products hi.hi + hi.lo +
// lo.hi accumulate in fp32 (x has no lo part when stored in bf16).  Theta is
// scaled by log2(e), so eta comes out in base-2 units for the MUFU ex2 / lg2.
// Each epilogue thread owns one chain, so the lp sum over rows stays in the
// thread (a compensated fp32 sum).
//
// The fp16 form (F16X3) runs the same products on fp16 hi/lo parts: 11 + 11
// significant bits per operand instead of 8 + 8, so the split represents each
// operand to about 2^-22 instead of 2^-17, at the same tensor-core rate.  The
// narrower fp16 exponent range is handled with exact power-of-two scales:
// X is stored times 2^sx (largest |x| in [2^13, 2^14), one sx per model),
// each chain's theta times 2^-e_c (largest |theta_k log2 e| in [2^13, 2^14),
// e_c computed with theta), the residual (|r| <= 1 for the logistic link)
// times 2^14; the epilogue multiplies eta by 2^(e_c - sx) and the gradient by
// 2^-(sx + 14).
//
// TMEM columns (512): eta^T [0, 128), G^T [128, 256), Theta hi [256, 320) and
// lo [320, 384), R hi [384, 448) and lo [448, 512).  Shared memory: a 3-stage
// ring of 128-row X tiles (hi + lo + y, 65 KiB each).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <math.h>

#include <string.h>

#include <algorithm>
#include <string>

#include "../../include/gbnuts.h"
#include "gbnuts_internal.h"
#include "tc_common.cuh"

namespace gbn {

using namespace tc;

namespace tct {

constexpr int TM = 128;            // rows per pre-tiled X tile
constexpr int TK = 128;            // features per tile (K + intercept, zero padded)
constexpr int NCH = 128;           // chains per CTA (TMEM lanes)
constexpr int PART_BYTES = TM * TK * 2;   // one bf16 part of an X tile
constexpr int Y_BYTES = TM * 4;
constexpr int STAGE_BYTES = 2 * PART_BYTES + 1024;  // X hi, X lo, y (padded)
constexpr int STAGES = 3;
constexpr int NUM_EPI_WARPS = 16;  // four per TMEM lane quarter
constexpr int EPI_SUB = NUM_EPI_WARPS / 4;
constexpr int RW = TM / EPI_SUB;   // rows of a pass per epilogue warp
constexpr int FW = TK / EPI_SUB;   // features per epilogue warp (gradient readout)
constexpr int THREADS = 64 + 32 * NUM_EPI_WARPS;
constexpr int SMEM_X = 0;
constexpr int SMEM_LP = SMEM_X + STAGES * STAGE_BYTES;   // [EPI_SUB][NCH] doubles
constexpr int SMEM_BAR = SMEM_LP + EPI_SUB * NCH * 8;
constexpr double kLn2 = 0.69314718055994530942;
constexpr int SMEM_TOTAL = SMEM_BAR + 256;
constexpr int SMEM_ALLOC = SMEM_TOTAL + 1024;  // slack for 1 KiB alignment
// TMEM column map
constexpr uint32_t COL_D1 = 0, COL_D2 = 128, COL_TH = 256, COL_TL = 320, COL_RH = 384,
                   COL_RL = 448;

// GEMM1 B operand: the 128 rows of a K-major tile part, features 16ks..16ks+15.
__device__ __forceinline__ uint64_t desc_rows(uint32_t part, int ks) {
  return make_desc(part + 256 * ks, 128, (TK / 8) * 128);
}
// GEMM2 B operand: the same part read MN-major (features x rows), rows
// 16ks..16ks+15.
__device__ __forceinline__ uint64_t desc_feats(uint32_t part, int ks) {
  return make_desc(part + 4096 * ks, (TK / 8) * 128, 128);
}

}  // namespace tct

struct TctArgs {
  const uint16_t* xt;  // pre-tiled X (16-bit hi/lo parts per 128-row tile)
  const float* yt;     // y per tile row
  long long N;
  int K, has_base, n_tiles;
  int x_exp;           // fp16 form: X is stored times 2^x_exp
  const double* Q;
  const uint32_t* QW;  // theta as packed words (kThetaWords per chain), or null
  int ldq, C;
  const int* active;
  double* P;
  int NP, S;
  int* err;
  // planned launch (a sampler run, active non-null): the plan is written
  // here ([0] splits, [1] slot stride, [2 + c] slot of chain c); null: the
  // grid is (S splits, chain groups) and chain c's partials are slot c
  int* dyn;
};

namespace tct {
// barrier slots (uint64 each) inside SMEM_BAR
enum { B_XFULL = 0, B_XEMPTY = 3, B_D1FULL = 6, B_D1EMPTY = 7, B_RFULL = 8, B_REMPTY = 9,
       B_D2FULL = 10, B_THETA = 11, B_COUNT = 12 };
}  // namespace tct

// Link terms of one pass for one chain: e2[j] = log2(e) eta of rows
// rr0 + j, y[j] their outcomes.  Accumulates pa, pb with lp = ln2 pa - pb
// (logistic: pa = sum y e2 - max(e2, 0) - log2(1 + 2^-|e2|), pb = 0;
// Poisson: pa = sum y e2, pb = sum mu) and packs r = y - mean as bf16 hi / lo
// pairs (F16: 2^14 r as fp16 hi / lo pairs).  MASK: rows j >= nvalid (past N)
// contribute nothing.
template <int LINK, bool MASK, int RWN, bool F16>
__device__ __forceinline__ void epilogue_values(const float* e2, const float* y, int nvalid,
                                                float& pa, float& pb, uint32_t* wh,
                                                uint32_t* wl) {
#pragma unroll
  for (int j = 0; j < RWN; j += 4) {
    const float4 y4 = *reinterpret_cast<const float4*>(y + j);
    const float yv[4] = {y4.x, y4.y, y4.z, y4.w};
    float res[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float x = e2[j + e];
      float ta, tb = 0.f, r;
      if (LINK == LINK_LOGIT) {
        const float ex = ex2_approx(-fabsf(x));
        const float d = 1.f + ex;
        const float inv = rcp_approx(d);
        const float sig = x >= 0.f ? inv : ex * inv;
        ta = yv[e] * x - fmaxf(x, 0.f) - lg2_approx(d);
        r = yv[e] - sig;
      } else {
        const float mu = ex2_approx(x);
        ta = yv[e] * x;
        tb = mu;
        r = yv[e] - mu;
      }
      if (MASK && j + e >= nvalid) {
        ta = 0.f;
        tb = 0.f;
        r = 0.f;
      }
      pa += ta;
      if (LINK != LINK_LOGIT) pb += tb;
      res[e] = r;
    }
#pragma unroll
    for (int e = 0; e < 4; e += 2) {
      if (F16) {
        const float r0 = res[e] * 16384.f, r1 = res[e + 1] * 16384.f;
        const __half2 hp = __floats2half2_rn(r0, r1);
        const float2 hf = __half22float2(hp);
        const __half2 lo = __floats2half2_rn(r0 - hf.x, r1 - hf.y);
        wh[(j + e) >> 1] = *reinterpret_cast<const uint32_t*>(&hp);
        wl[(j + e) >> 1] = *reinterpret_cast<const uint32_t*>(&lo);
      } else {
        const __nv_bfloat162 hp = __floats2bfloat162_rn(res[e], res[e + 1]);
        const float2 hf = __bfloat1622float2(hp);
        const __nv_bfloat162 lo = __floats2bfloat162_rn(res[e] - hf.x, res[e + 1] - hf.y);
        wh[(j + e) >> 1] = *reinterpret_cast<const uint32_t*>(&hp);
        wl[(j + e) >> 1] = *reinterpret_cast<const uint32_t*>(&lo);
      }
    }
  }
}

// s += v as an unevaluated fp32 pair (s.x + s.y), Knuth's two-sum.
__device__ __forceinline__ void two_sum_add(float2& s, float v) {
  const float t = s.x + v;
  const float bp = t - s.x;
  const float err = (s.x - (t - bp)) + (v - bp);
  s.x = t;
  s.y += err;
}

// SPLIT: the hi/lo split products (bf16x3); otherwise one bf16 product per
// contraction (the plain bf16 form; X's lo part unused).  F16: fp16 operands
// with the scales described above (used with XLO and SPLIT).
template <int LINK, bool XLO, bool SPLIT, bool F16>
__global__ void __launch_bounds__(tct::THREADS, 1) glm_tct_kernel(TctArgs a) {
  using namespace tct;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  double* sLP = reinterpret_cast<double*>(sm + SMEM_LP);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + SMEM_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SMEM_BAR + 8 * B_COUNT);
  volatile int* abort_s = reinterpret_cast<volatile int*>(sm + SMEM_BAR + 8 * B_COUNT + 8);
  __shared__ int act_s[NCH];
  __shared__ int chain_s[NCH];  // chain of each TMEM lane (M row)

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int hb = a.has_base;
  const int Kx = a.K + hb;

  // This CTA's row split s of S_eff, and its chain group gs: lanes
  // 0..127 hold the chains of slots 128 gs .. 128 gs + 127, whose partials
  // are rows s * slot_stride + slot of P.
  int s, S_eff, gs;
  size_t slot_stride;
  if (a.dyn) {
    // Planned: the chains requesting a gradient, in chain order, fill slots
    // 0..n_act-1; the grid's CTAs are spread over their ceil(n_act / 128)
    // groups.  Every CTA derives the same plan from the active flags.
    __shared__ uint32_t bits_s[kTctPlanMaxChains / 32];
    __shared__ int pre_s[kTctPlanMaxChains / 32 + 1];
    const int W = (a.C + 31) / 32;
    for (int w = warp; w < W; w += THREADS / 32) {
      const int cg = 32 * w + lane;
      const unsigned on = __ballot_sync(0xffffffffu, cg < a.C && a.active[cg] != 0);
      if (lane == 0) bits_s[w] = on;
    }
    __syncthreads();
    if (warp == 0) {
      // exclusive prefix of the words' active counts
      int run = 0;
      for (int w0 = 0; w0 < W; w0 += 32) {
        const int w = w0 + lane;
        const int cnt = w < W ? __popc(bits_s[w]) : 0;
        int incl = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, incl, off);
          if (lane >= off) incl += v;
        }
        if (w < W) pre_s[w] = run + incl - cnt;
        run += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (lane == 0) pre_s[W] = run;
    }
    __syncthreads();
    const int n_act = pre_s[W];
    if (n_act == 0) return;
    const int g_act = (n_act + NCH - 1) / NCH;
    S_eff = min(max(1, (int)gridDim.x / g_act), a.n_tiles);
    gs = (int)blockIdx.x / S_eff;
    s = (int)blockIdx.x - gs * S_eff;
    if (gs >= g_act) return;
    slot_stride = (size_t)NCH * g_act;
    if (tid < NCH) {
      const int slot = NCH * gs + tid;
      int chain = 0, on = 0;
      if (slot < n_act) {
        // the word holding active chain #slot, then its bit
        int lo = 0, hi = W - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (pre_s[mid] <= slot)
            lo = mid;
          else
            hi = mid - 1;
        }
        uint32_t bb = bits_s[lo];
        for (int j = slot - pre_s[lo]; j > 0; --j) bb &= bb - 1;
        chain = 32 * lo + __ffs(bb) - 1;
        on = 1;
        if (s == 0) a.dyn[2 + chain] = slot;
      }
      act_s[tid] = on;
      chain_s[tid] = chain;
    }
    if (blockIdx.x == 0 && tid == 0) {
      a.dyn[0] = S_eff;
      a.dyn[1] = (int)slot_stride;
    }
    __syncthreads();
  } else {
    s = blockIdx.x;
    S_eff = a.S;
    gs = blockIdx.y;
    slot_stride = (size_t)a.C;
    if (tid < NCH) {
      const int cg = NCH * gs + tid;
      act_s[tid] = (cg < a.C) && (a.active == nullptr || a.active[cg] != 0);
      chain_s[tid] = cg < a.C ? cg : 0;
    }
    const int any = __syncthreads_or(tid < NCH ? act_s[tid] : 0);
    if (!any) return;
  }
  const size_t row0_slot = (size_t)NCH * gs;  // slot of lane 0

  if (tid == 0) {
    for (int b = 0; b < STAGES; ++b) {
      mbar_init(&bars[B_XFULL + b], 1);
      mbar_init(&bars[B_XEMPTY + b], 1);
    }
    mbar_init(&bars[B_D1FULL], 1);
    mbar_init(&bars[B_D1EMPTY], NUM_EPI_WARPS);
    mbar_init(&bars[B_RFULL], NUM_EPI_WARPS);
    mbar_init(&bars[B_REMPTY], 1);
    mbar_init(&bars[B_D2FULL], 1);
    mbar_init(&bars[B_THETA], NUM_EPI_WARPS);
    *abort_s = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, 512);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  const int t_begin = (int)((long long)a.n_tiles * s / S_eff);
  const int t_end = (int)((long long)a.n_tiles * (s + 1) / S_eff);
  const int n = t_end - t_begin;
  constexpr bool kXlo = XLO && SPLIT;
  const uint32_t x_bytes = kXlo ? 2u * PART_BYTES : (uint32_t)PART_BYTES;
  const int ksteps = (Kx + 15) / 16;   // GEMM1 contraction steps holding features
  const int nf = 16 * ksteps;          // GEMM2 N: features rounded up to 16

  if (n > 0) {
    if (warp == 0) {
      // ---- producer: X tiles through the 3-stage ring
      if (lane == 0) {
        for (int i = 0; i < n; ++i) {
          const int st = i % STAGES, u = i / STAGES;
          if (!mbar_wait_abortable(&bars[B_XEMPTY + st], (u & 1) ^ 1, abort_s, a.err, 21)) break;
          unsigned char* dst = sm + SMEM_X + st * STAGE_BYTES;
          const uint16_t* src = a.xt + (size_t)(2 * (t_begin + i)) * (TM * TK);
          mbar_arrive_expect_tx(&bars[B_XFULL + st], x_bytes + Y_BYTES);
          bulk_copy_g2s(dst, src, PART_BYTES, &bars[B_XFULL + st]);
          if (kXlo)
            bulk_copy_g2s(dst + PART_BYTES, src + TM * TK, PART_BYTES, &bars[B_XFULL + st]);
          bulk_copy_g2s(dst + 2 * PART_BYTES, a.yt + (size_t)(t_begin + i) * TM, Y_BYTES,
                        &bars[B_XFULL + st]);
        }
      }
      __syncwarp();
    } else if (warp == 1) {
      // ---- MMA issuer: GEMM1 of tile i, then GEMM2 of tile i - 1
      if (lane == 0) {
        const uint32_t id1 = make_idesc_bf16(NCH, TM, 0, 0, F16);
        const uint32_t id2 = make_idesc_bf16(NCH, nf, 0, 1, F16);
        bool ok = mbar_wait_abortable(&bars[B_THETA], 0, abort_s, a.err, 22);
        fence_after_sync();
        auto gemm2 = [&](int i) -> bool {
          if (!mbar_wait_abortable(&bars[B_RFULL], i & 1, abort_s, a.err, 23)) return false;
          fence_after_sync();
          const int st = i % STAGES;
          const uint32_t xh = smem_u32(sm + SMEM_X + st * STAGE_BYTES);
          // descriptors advance by their start-address field (16-byte units);
          // few instructions per MMA, as the issuing warp shares its
          // scheduler with four epilogue warps
          const uint64_t bh0 = desc_feats(xh, 0), bl0 = desc_feats(xh + PART_BYTES, 0);
          const uint32_t drow = tmem + COL_D2, arh = tmem + COL_RH, arl = tmem + COL_RL;
          mma_bf16_tmem_a(drow, arh, bh0, id2, i > 0 ? 1u : 0u);
          if (SPLIT) mma_bf16_tmem_a(drow, arl, bh0, id2, 1u);
          if (kXlo) mma_bf16_tmem_a(drow, arh, bl0, id2, 1u);
#pragma unroll
          for (int ks = 1; ks < TM / 16; ++ks) {
            const uint64_t bh = bh0 + (uint64_t)(256 * ks);
            mma_bf16_tmem_a(drow, arh + 8 * ks, bh, id2, 1u);
            if (SPLIT) mma_bf16_tmem_a(drow, arl + 8 * ks, bh, id2, 1u);
            if (kXlo) mma_bf16_tmem_a(drow, arh + 8 * ks, bl0 + (uint64_t)(256 * ks), id2, 1u);
          }
          mma_commit(&bars[B_REMPTY]);
          mma_commit(&bars[B_XEMPTY + st]);
          return true;
        };
        for (int i = 0; i < n && ok; ++i) {
          const int st = i % STAGES;
          ok = mbar_wait_abortable(&bars[B_XFULL + st], (i / STAGES) & 1, abort_s, a.err, 24) &&
               mbar_wait_abortable(&bars[B_D1EMPTY], (i & 1) ^ 1, abort_s, a.err, 25);
          if (!ok) break;
          fence_after_sync();
          const uint32_t xh = smem_u32(sm + SMEM_X + st * STAGE_BYTES);
          const uint64_t bh0 = desc_rows(xh, 0), bl0 = desc_rows(xh + PART_BYTES, 0);
          const uint32_t d1 = tmem + COL_D1, ath = tmem + COL_TH, atl = tmem + COL_TL;
          mma_bf16_tmem_a(d1, ath, bh0, id1, 0u);
          if (SPLIT) mma_bf16_tmem_a(d1, atl, bh0, id1, 1u);
          if (kXlo) mma_bf16_tmem_a(d1, ath, bl0, id1, 1u);
#pragma unroll 1
          for (int ks = 1; ks < ksteps; ++ks) {
            const uint64_t bh = bh0 + (uint64_t)(16 * ks);
            mma_bf16_tmem_a(d1, ath + 8 * ks, bh, id1, 1u);
            if (SPLIT) mma_bf16_tmem_a(d1, atl + 8 * ks, bh, id1, 1u);
            if (kXlo) mma_bf16_tmem_a(d1, ath + 8 * ks, bl0 + (uint64_t)(16 * ks), id1, 1u);
          }
          mma_commit(&bars[B_D1FULL]);
          if (i > 0) ok = gemm2(i - 1);
        }
        if (ok) ok = gemm2(n - 1);
        mma_commit(&bars[B_D2FULL]);
        // no MMA may still run when tensor memory is released
        mbar_wait(&bars[B_D2FULL], 0, a.err, 29);
      }
      __syncwarp();
    } else {
      // ---- epilogue: warp w owns TMEM lane quarter q = w % 4 (chains
      // 32q..32q+31), rows RW*sub.. of every tile and features FW*sub..
      const int q = warp & 3;
      const int sub = (warp - 2) >> 2;
      const int c = 32 * q + lane;
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
      // log2(e) Theta of this chain -> TMEM as bf16 hi / lo pairs (fp32 split),
      // or for F16 as fp16 hi / lo pairs at the chain's scale 2^-e_c
      float eta_scale = 1.f;
      {
        const bool act = act_s[c] != 0;
        const double* th = a.Q + (size_t)(act ? chain_s[c] : 0) * a.ldq;
        const uint32_t* tw = a.QW ? a.QW + (size_t)(act ? chain_s[c] : 0) * kThetaWords : nullptr;
        int e_c = 0;
        if (F16 && act) {
          if (tw) {
            e_c = (int)tw[kThetaExpWord];
          } else {
            float fmax = 0.f;
            for (int k = 0; k < Kx; ++k) fmax = fmaxf(fmax, fabsf(theta_f32(th[k])));
            e_c = theta_exp_f16(fmax);
          }
          const int es = max(-126, min(126, e_c - a.x_exp));
          eta_scale = exp2_int(es);
        }
        const float th_scale = exp2_int(-e_c);
#pragma unroll
        for (int part = 0; part < FW / 32; ++part) {
          uint32_t wh[16], wl[16];
          const int w0 = FW / 2 * sub + 16 * part;
          if (tw && act) {
            // words written by the step kernel with the request (vector loads)
#pragma unroll
            for (int j = 0; j < 16; j += 4) {
              const uint4 h4 = *reinterpret_cast<const uint4*>(tw + w0 + j);
              const uint4 l4 = *reinterpret_cast<const uint4*>(tw + 64 + w0 + j);
              wh[j] = h4.x; wh[j + 1] = h4.y; wh[j + 2] = h4.z; wh[j + 3] = h4.w;
              wl[j] = l4.x; wl[j + 1] = l4.y; wl[j + 2] = l4.z; wl[j + 3] = l4.w;
            }
          } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int k = FW * sub + 32 * part + 2 * j;
              const double d0 = (act && k < Kx) ? th[k] : 0.0;
              const double d1 = (act && k + 1 < Kx) ? th[k + 1] : 0.0;
              if (F16)
                theta_words_f16(theta_f32(d0), theta_f32(d1), th_scale, wh[j], wl[j]);
              else
                theta_words(d0, d1, wh[j], wl[j]);
            }
          }
          tmem_st16(lane_addr + COL_TH + FW / 2 * sub + 16 * part, wh);
          tmem_st16(lane_addr + COL_TL + FW / 2 * sub + 16 * part, wl);
        }
        tmem_st_wait();
        fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_THETA]);
      }
      float2 sa = make_float2(0.f, 0.f), sb = make_float2(0.f, 0.f);  // compensated
      bool ok = true;
      for (int i = 0; i < n && ok; ++i) {
        const int st = i % STAGES;
        if (!warp_wait(&bars[B_D1FULL], i & 1, abort_s, a.err, 26)) {
          ok = false;
          break;
        }
        fence_after_sync();
        float v[RW];
        tmem_ld32(lane_addr + COL_D1 + RW * sub, v);
        tmem_ld_wait();
        if (F16) {
#pragma unroll
          for (int j = 0; j < RW; ++j) v[j] *= eta_scale;
        }
        fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_D1EMPTY]);
        const int rr0 = RW * sub;
        const float* ys =
            reinterpret_cast<const float*>(sm + SMEM_X + st * STAGE_BYTES + 2 * PART_BYTES) + rr0;
        const long long row0 = (long long)(t_begin + i) * TM + rr0;
        const int nvalid = (int)max(0LL, min((long long)RW, a.N - row0));
        float pa = 0.f, pb = 0.f;
        uint32_t wh[RW / 2], wl[RW / 2];
        if (nvalid == RW)
          epilogue_values<LINK, false, RW, F16>(v, ys, RW, pa, pb, wh, wl);
        else
          epilogue_values<LINK, true, RW, F16>(v, ys, nvalid, pa, pb, wh, wl);
        two_sum_add(sa, pa);
        if (LINK != LINK_LOGIT) two_sum_add(sb, pb);
        if (!warp_wait(&bars[B_REMPTY], (i & 1) ^ 1, abort_s, a.err, 27)) {
          ok = false;
          break;
        }
        fence_after_sync();
        tmem_st16(lane_addr + COL_RH + RW / 2 * sub, wh);
        tmem_st16(lane_addr + COL_RL + RW / 2 * sub, wl);
        tmem_st_wait();
        fence_before_sync();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_RFULL]);
      }
      sLP[sub * NCH + c] =
          kLn2 * ((double)sa.x + (double)sa.y) - ((double)sb.x + (double)sb.y);
      // gradient partials: this chain's features FW*sub .. FW*sub + FW - 1
      if (ok && warp_wait(&bars[B_D2FULL], 0, abort_s, a.err, 28)) {
        fence_after_sync();
        float g[FW];
#pragma unroll
        for (int j = 0; j < FW; j += 32) tmem_ld32(lane_addr + COL_D2 + FW * sub + j, g + j);
        tmem_ld_wait();
        if (F16) {
          const float gs = exp2_int(max(-126, min(126, -a.x_exp - 14)));
#pragma unroll
          for (int j = 0; j < FW; ++j) g[j] *= gs;
        }
        if (act_s[c]) {
          double* dst = a.P + ((size_t)s * slot_stride + row0_slot + c) * a.NP;
#pragma unroll
          for (int j = 0; j < FW; ++j) {
            const int k = FW * sub + j;
            if (k < hb)
              dst[1] = (double)g[j];
            else if (k < Kx)
              dst[4 + (k - hb)] = (double)g[j];
          }
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid < NCH && act_s[tid]) {
    double* dst = a.P + ((size_t)s * slot_stride + row0_slot + tid) * a.NP;
    double lp = 0.0;
    if (n > 0)
      for (int k = 0; k < EPI_SUB; ++k) lp += sLP[k * NCH + tid];
    dst[0] = lp;
    dst[2] = 0.0;
    dst[3] = 0.0;
    if (n == 0) {
      for (int k = 0; k < Kx; ++k) dst[k < hb ? 1 : 4 + (k - hb)] = 0.0;
    }
  }
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, 512);
  }
}

int tct_plan_grid(int C) {
  return std::max(device_sm_count(), (C + tct::NCH - 1) / tct::NCH);
}

int tct_splits(const ModelDesc& m, int C) {
  const int groups = (C + tct::NCH - 1) / tct::NCH;
  int S = std::max(1, device_sm_count() / groups);
  S = std::min<long long>(S, std::max(1, m.tc_tiles));
  return S;
}

// ------------------------------------------------------------------ tiles
// X as 128-row tiles, each a hi part then a lo part of 128 x 128 16-bit
// values in the canonical K-major core-matrix layout (feature 0 is the
// intercept's constant 1 when the model has one), and y per tile row.
// F16: the parts are fp16 of x 2^x_exp; otherwise bf16 of x.
template <bool F16>
__global__ void tct_tiles_kernel(const void* X, int x_dtype, long long N, int K, int has_base,
                                 int n_tiles, uint16_t* xt, float scale) {
  using namespace tct;
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
    uint16_t hb, lb;
    if (F16) {
      __half hi, lo;
      split_f16(v * scale, hi, lo);
      hb = __half_as_ushort(hi);
      lb = __half_as_ushort(lo);
    } else {
      __nv_bfloat16 hi, lo;
      split_bf16(v, hi, lo);
      hb = __bfloat16_as_ushort(hi);
      lb = __bfloat16_as_ushort(lo);
    }
    const uint32_t off = kmajor_off(r, k, TK) / 2;
    xt[(2 * t) * (TM * TK) + off] = hb;
    xt[(2 * t + 1) * (TM * TK) + off] = lb;
  }
}

__global__ void tct_y_kernel(long long N, int n_tiles, const double* y, float* yt) {
  const long long total = (long long)n_tiles * tct::TM;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x)
    yt[i] = i < N ? (float)y[i] : 0.f;
}

// Largest |x| of the design (as fp32 bits; non-negative floats order like
// their bit patterns).
__global__ void tct_maxabs_kernel(const void* X, int x_dtype, long long n, unsigned* out) {
  float mx = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float v;
    if (x_dtype == GBNUTS_F64)
      v = (float)static_cast<const double*>(X)[i];
    else if (x_dtype == GBNUTS_F32)
      v = static_cast<const float*>(X)[i];
    else
      v = __uint_as_float(((unsigned)static_cast<const uint16_t*>(X)[i]) << 16);
    mx = fmaxf(mx, fabsf(v));
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(mx));
}

int tc_prepare(const ModelDesc& m, bool f16, void** xt, float** yt, int* n_tiles, int* x_exp,
               cudaStream_t st) {
  using namespace tct;
  const int tiles = (int)((m.N + TM - 1) / TM);
  const size_t xbytes = (size_t)tiles * 2 * PART_BYTES;
  const int threads = 256;
  const int grid_cap = device_sm_count() * 16;
  float scale = 1.f;
  *x_exp = 0;
  if (f16) {
    // x_exp: the largest |x| (and the intercept's 1) times 2^x_exp in [2^13, 2^14)
    unsigned* d_mx = nullptr;
    GBN_CUDA_TRY(cudaMalloc(&d_mx, sizeof(unsigned)));
    GBN_CUDA_TRY(cudaMemsetAsync(d_mx, 0, sizeof(unsigned), st));
    const long long n = m.N * (long long)m.K;
    if (n > 0)
      tct_maxabs_kernel<<<(int)std::min<long long>((n + threads - 1) / threads, grid_cap), threads,
                          0, st>>>(m.X, m.x_dtype, n, d_mx);
    unsigned bits = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, d_mx, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_mx);
    if (e != cudaSuccess) {
      set_last_error(std::string("design range: ") + cudaGetErrorString(e));
      return GBNUTS_SOFTWARE;
    }
    float mx = 0.f;
    memcpy(&mx, &bits, sizeof(float));
    if (m.has_base) mx = std::max(mx, 1.f);
    if (!(mx < 3.0e38f)) {
      set_last_error("the fp16 form needs a finite design matrix");
      return GBNUTS_DATAERR;
    }
    if (mx > 0.f) {
      int e2 = 0;
      frexpf(mx, &e2);
      *x_exp = std::max(-100, std::min(100, 13 - (e2 - 1)));
    }
    scale = ldexpf(1.f, *x_exp);
  }
  GBN_CUDA_TRY(cudaMalloc(xt, xbytes));
  const long long total = (long long)tiles * TM * TK;
  const int blocks = (int)std::min<long long>((total + threads - 1) / threads, grid_cap);
  if (f16)
    tct_tiles_kernel<true><<<blocks, threads, 0, st>>>(m.X, m.x_dtype, m.N, m.K, m.has_base,
                                                       tiles, static_cast<uint16_t*>(*xt), scale);
  else
    tct_tiles_kernel<false><<<blocks, threads, 0, st>>>(m.X, m.x_dtype, m.N, m.K, m.has_base,
                                                        tiles, static_cast<uint16_t*>(*xt), scale);
  GBN_CUDA_TRY(cudaGetLastError());
  if (*yt == nullptr) {
    GBN_CUDA_TRY(cudaMalloc(yt, (size_t)tiles * TM * sizeof(float)));
    tct_y_kernel<<<std::max(1, std::min(grid_cap, (tiles * TM + threads - 1) / threads)), threads,
                   0, st>>>(m.N, tiles, m.y, *yt);
    GBN_CUDA_TRY(cudaGetLastError());
  }
  *n_tiles = tiles;
  return GBNUTS_OK;
}

template <int LINK, bool XLO, bool SPLIT, bool F16>
static int launch_tct_t(const TctArgs& a, dim3 grid, cudaStream_t st) {
  using namespace tct;
  int rc = ensure_smem(glm_tct_kernel<LINK, XLO, SPLIT, F16>, SMEM_ALLOC);
  if (rc) return rc;
  glm_tct_kernel<LINK, XLO, SPLIT, F16><<<grid, THREADS, SMEM_ALLOC, st>>>(a);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

int launch_tct(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
               const int* active, GradWorkspace& ws, cudaStream_t st) {
  using namespace tct;
  const bool f16 = precision == GBNUTS_PREC_F16X3;
  TctArgs a;
  a.xt = static_cast<const uint16_t*>(f16 ? m.tc_xt16 : m.tc_xt);
  a.yt = m.tc_yt;
  a.N = m.N;
  a.K = m.K;
  a.has_base = m.has_base;
  a.n_tiles = m.tc_tiles;
  a.x_exp = m.tc_x_exp;
  a.Q = Q;
  a.QW = ws.tc_words;
  a.ldq = ldq;
  a.C = C;
  a.active = active;
  a.P = ws.partial;
  a.NP = ws.NP;
  a.S = ws.S;
  a.err = ws.err;
  const bool planned = active != nullptr && ws.dyn != nullptr && tct_dynamic(m, precision, C);
  a.dyn = planned ? ws.dyn : nullptr;
  if (a.xt == nullptr || a.yt == nullptr) {
    set_last_error("tensor-core tiles of X are not prepared for this precision");
    return GBNUTS_SOFTWARE;
  }
  const bool xlo = m.x_dtype != GBNUTS_BF16;
  const bool split = precision == GBNUTS_PREC_BF16X3;
  dim3 grid = planned ? dim3(tct_plan_grid(C)) : dim3(ws.S, (C + NCH - 1) / NCH);
  if (f16) {
    if (m.link != LINK_LOGIT) {
      set_last_error("the f16x3 form takes the logistic GLM");
      return GBNUTS_USAGE;
    }
    return launch_tct_t<LINK_LOGIT, true, true, true>(a, grid, st);
  }
  if (m.link == LINK_LOGIT) {
    if (!split) return launch_tct_t<LINK_LOGIT, false, false, false>(a, grid, st);
    return xlo ? launch_tct_t<LINK_LOGIT, true, true, false>(a, grid, st)
               : launch_tct_t<LINK_LOGIT, false, true, false>(a, grid, st);
  }
  if (!split) return launch_tct_t<LINK_POISSON_LOG, false, false, false>(a, grid, st);
  return xlo ? launch_tct_t<LINK_POISSON_LOG, true, true, false>(a, grid, st)
             : launch_tct_t<LINK_POISSON_LOG, false, true, false>(a, grid, st);
}

// ------------------------------------------------------------------ probe
// Checks the tensor-memory A operand and both B layouts on one tile:
// D1 = A . X^T (A: 128 x 128 in TMEM from Aw, X: 128 rows x 128 features),
// D2 = R . X   (R: 128 x 128 rows in TMEM from Rw).  Aw, Rw: 128 lanes x 64
// 32-bit words each, written to TMEM as given.
__global__ void __launch_bounds__(128, 1)
    tct_probe_kernel(const uint32_t* Aw, const __nv_bfloat16* X, const uint32_t* Rw, float* D1,
                     float* D2, int* err) {
  using namespace tct;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  unsigned char* sX = sm;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + PART_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + PART_BYTES + 16);
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < TM * TK; i += 128) {
    const int r = i / TK, k = i - r * TK;
    *reinterpret_cast<__nv_bfloat16*>(sX + kmajor_off(r, k, TK)) = X[i];
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, 512);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  for (int j = 0; j < 64; j += 16) {
    uint32_t a[16], r[16];
    for (int i = 0; i < 16; ++i) {
      a[i] = Aw[tid * 64 + j + i];
      r[i] = Rw[tid * 64 + j + i];
    }
    tmem_st16(lane_base + 256 + j, a);
    tmem_st16(lane_base + 320 + j, r);
  }
  tmem_st_wait();
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (tid == 0) {
    const uint32_t sx = smem_u32(sX);
    const uint32_t id1 = make_idesc_bf16(128, 128, 0, 0);
    const uint32_t id2 = make_idesc_bf16(128, 128, 0, 1);
    for (int ks = 0; ks < TK / 16; ++ks)
      mma_bf16_tmem_a(tmem + 0, tmem + 256 + 8 * ks, desc_rows(sx, ks), id1, ks > 0);
    for (int ks = 0; ks < TM / 16; ++ks)
      mma_bf16_tmem_a(tmem + 128, tmem + 320 + 8 * ks, desc_feats(sx, ks), id2, ks > 0);
    mma_commit(bar);
  }
  const bool ok = mbar_wait(bar, 0, err, 3);
  fence_after_sync();
  if (ok) {
    float v[32];
    for (int j = 0; j < 128; j += 32) {
      tmem_ld32(lane_base + j, v);
      tmem_ld_wait();
      for (int c = 0; c < 32; ++c) D1[tid * 128 + j + c] = v[c];
      tmem_ld32(lane_base + 128 + j, v);
      tmem_ld_wait();
      for (int c = 0; c < 32; ++c) D2[tid * 128 + j + c] = v[c];
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, 512);
  }
}

// A wait that nothing satisfies, bounded by `limit` cycles (test hook).
__global__ void wait_probe_kernel(long long limit, int* err, int* completed) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
    *completed = tc::mbar_wait_limit(&bar, 0, limit, err, 77) ? 1 : 0;
  }
}

}  // namespace gbn

extern "C" int gbnuts_wait_probe(long long limit_cycles, int* code, int* completed) {
  using namespace gbn;
  if (limit_cycles <= 0 || limit_cycles > 8000000000LL || !code || !completed) {
    set_last_error("wait probe: limit_cycles in (0, 8e9] and non-null outputs");
    return GBNUTS_USAGE;
  }
  int* d = nullptr;
  GBN_CUDA_TRY(cudaMalloc(&d, 2 * sizeof(int)));
  GBN_CUDA_TRY(cudaMemset(d, 0, 2 * sizeof(int)));
  wait_probe_kernel<<<1, 32>>>(limit_cycles, d, d + 1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_last_error(std::string("wait probe: ") + cudaGetErrorString(e));
    return GBNUTS_SOFTWARE;
  }
  *code = h[0];
  *completed = h[1];
  return GBNUTS_OK;
}

// Test hook (include/gbnuts_testing.h): runs the probe kernel on host arrays.
extern "C" int gbnuts_tct_probe(const uint32_t* Aw, const uint16_t* X, const uint32_t* Rw,
                                float* D1, float* D2) {
  using namespace gbn;
  using namespace gbn::tct;
  void *dA, *dX, *dR, *dD1, *dD2, *dE;
  GBN_CUDA_TRY(cudaMalloc(&dA, 128 * 64 * 4));
  GBN_CUDA_TRY(cudaMalloc(&dX, TM * TK * 2));
  GBN_CUDA_TRY(cudaMalloc(&dR, 128 * 64 * 4));
  GBN_CUDA_TRY(cudaMalloc(&dD1, 128 * 128 * 4));
  GBN_CUDA_TRY(cudaMalloc(&dD2, 128 * 128 * 4));
  GBN_CUDA_TRY(cudaMalloc(&dE, 4));
  GBN_CUDA_TRY(cudaMemset(dE, 0, 4));
  GBN_CUDA_TRY(cudaMemcpy(dA, Aw, 128 * 64 * 4, cudaMemcpyHostToDevice));
  GBN_CUDA_TRY(cudaMemcpy(dX, X, TM * TK * 2, cudaMemcpyHostToDevice));
  GBN_CUDA_TRY(cudaMemcpy(dR, Rw, 128 * 64 * 4, cudaMemcpyHostToDevice));
  const int smem = PART_BYTES + 64 + 1024;
  GBN_CUDA_TRY(cudaFuncSetAttribute(tct_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem));
  tct_probe_kernel<<<1, 128, smem>>>((const uint32_t*)dA, (const __nv_bfloat16*)dX,
                                     (const uint32_t*)dR, (float*)dD1, (float*)dD2, (int*)dE);
  GBN_CUDA_TRY(cudaGetLastError());
  GBN_CUDA_TRY(cudaDeviceSynchronize());
  int e = 0;
  GBN_CUDA_TRY(cudaMemcpy(&e, dE, 4, cudaMemcpyDeviceToHost));
  GBN_CUDA_TRY(cudaMemcpy(D1, dD1, 128 * 128 * 4, cudaMemcpyDeviceToHost));
  GBN_CUDA_TRY(cudaMemcpy(D2, dD2, 128 * 128 * 4, cudaMemcpyDeviceToHost));
  cudaFree(dA);
  cudaFree(dX);
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
