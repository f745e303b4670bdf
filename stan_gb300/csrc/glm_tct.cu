// Batched GLM log density and gradient on the tcgen05 tensor cores, chains on
// the M dimension (precision GBNUTS_PREC_BF16X3, logistic and Poisson).
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
// TMEM columns (512): eta^T [0, 128), G^T [128, 256), Theta hi [256, 320) and
// lo [320, 384), R hi [384, 448) and lo [448, 512).  Shared memory: a 3-stage
// ring of 128-row X tiles (hi + lo + y, 65 KiB each).
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>

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
  const __nv_bfloat16* xt;  // pre-tiled X (hi/lo per 128-row tile)
  const float* yt;          // y per tile row
  long long N;
  int K, has_base, n_tiles;
  const double* Q;
  const uint32_t* QW;  // theta as packed words (kThetaWords per chain), or null
  int ldq, C;
  const int* active;
  double* P;
  int NP, S;
  int* err;
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
// pairs.  MASK: rows j >= nvalid (past N) contribute nothing.
template <int LINK, bool MASK, int RWN>
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
      const __nv_bfloat162 hp = __floats2bfloat162_rn(res[e], res[e + 1]);
      const float2 hf = __bfloat1622float2(hp);
      const __nv_bfloat162 lo = __floats2bfloat162_rn(res[e] - hf.x, res[e + 1] - hf.y);
      wh[(j + e) >> 1] = *reinterpret_cast<const uint32_t*>(&hp);
      wl[(j + e) >> 1] = *reinterpret_cast<const uint32_t*>(&lo);
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
// contraction (the plain bf16 form; X's lo part unused).
template <int LINK, bool XLO, bool SPLIT>
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

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s = blockIdx.x;
  const int c0 = blockIdx.y * NCH;
  const int hb = a.has_base;
  const int Kx = a.K + hb;

  if (tid < NCH) {
    const int cg = c0 + tid;
    act_s[tid] = (cg < a.C) && (a.active == nullptr || a.active[cg] != 0);
  }
  const int any = __syncthreads_or(tid < NCH ? act_s[tid] : 0);
  if (!any) return;

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

  const int t_begin = (int)((long long)a.n_tiles * s / a.S);
  const int t_end = (int)((long long)a.n_tiles * (s + 1) / a.S);
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
          const __nv_bfloat16* src = a.xt + (size_t)(2 * (t_begin + i)) * (TM * TK);
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
        const uint32_t id1 = make_idesc_bf16(NCH, TM, 0, 0);
        const uint32_t id2 = make_idesc_bf16(NCH, nf, 0, 1);
        bool ok = mbar_wait_abortable(&bars[B_THETA], 0, abort_s, a.err, 22);
        fence_after_sync();
        auto gemm2 = [&](int i) -> bool {
          if (!mbar_wait_abortable(&bars[B_RFULL], i & 1, abort_s, a.err, 23)) return false;
          fence_after_sync();
          const int st = i % STAGES;
          const uint32_t xh = smem_u32(sm + SMEM_X + st * STAGE_BYTES);
          const uint32_t xl = xh + PART_BYTES;
#pragma unroll 1
          for (int ks = 0; ks < TM / 16; ++ks) {
            const uint64_t bh = desc_feats(xh, ks);
            mma_bf16_tmem_a(tmem + COL_D2, tmem + COL_RH + 8 * ks, bh, id2,
                            (i > 0 || ks > 0) ? 1u : 0u);
            if (SPLIT) mma_bf16_tmem_a(tmem + COL_D2, tmem + COL_RL + 8 * ks, bh, id2, 1u);
            if (kXlo) mma_bf16_tmem_a(tmem + COL_D2, tmem + COL_RH + 8 * ks, desc_feats(xl, ks), id2, 1u);
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
          const uint32_t xl = xh + PART_BYTES;
#pragma unroll 1
          for (int ks = 0; ks < ksteps; ++ks) {
            const uint64_t bh = desc_rows(xh, ks);
            mma_bf16_tmem_a(tmem + COL_D1, tmem + COL_TH + 8 * ks, bh, id1, ks > 0 ? 1u : 0u);
            if (SPLIT) mma_bf16_tmem_a(tmem + COL_D1, tmem + COL_TL + 8 * ks, bh, id1, 1u);
            if (kXlo) mma_bf16_tmem_a(tmem + COL_D1, tmem + COL_TH + 8 * ks, desc_rows(xl, ks), id1, 1u);
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
      // log2(e) Theta of this chain -> TMEM as bf16 hi / lo pairs (fp32 split)
      {
        const bool act = act_s[c] != 0;
        const double* th = a.Q + (size_t)(act ? c0 + c : 0) * a.ldq;
        const uint32_t* tw = a.QW ? a.QW + (size_t)(act ? c0 + c : 0) * kThetaWords : nullptr;
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
              theta_words((act && k < Kx) ? th[k] : 0.0, (act && k + 1 < Kx) ? th[k + 1] : 0.0,
                          wh[j], wl[j]);
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
          epilogue_values<LINK, false, RW>(v, ys, RW, pa, pb, wh, wl);
        else
          epilogue_values<LINK, true, RW>(v, ys, nvalid, pa, pb, wh, wl);
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
        if (act_s[c]) {
          double* dst = a.P + ((size_t)s * a.C + c0 + c) * a.NP;
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
    double* dst = a.P + ((size_t)s * a.C + c0 + tid) * a.NP;
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

int tct_splits(const ModelDesc& m, int C) {
  const int groups = (C + tct::NCH - 1) / tct::NCH;
  int S = std::max(1, 148 / groups);
  S = std::min<long long>(S, std::max(1, m.tc_tiles));
  return S;
}

template <int LINK, bool XLO, bool SPLIT>
static int launch_tct_t(const TctArgs& a, dim3 grid, cudaStream_t st) {
  using namespace tct;
  static bool attr = false;
  if (!attr) {
    GBN_CUDA_TRY(cudaFuncSetAttribute(glm_tct_kernel<LINK, XLO, SPLIT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_ALLOC));
    attr = true;
  }
  glm_tct_kernel<LINK, XLO, SPLIT><<<grid, THREADS, SMEM_ALLOC, st>>>(a);
  GBN_CUDA_TRY(cudaGetLastError());
  return GBNUTS_OK;
}

int launch_tct(const ModelDesc& m, int precision, const double* Q, int ldq, int C,
               const int* active, GradWorkspace& ws, cudaStream_t st) {
  using namespace tct;
  TctArgs a;
  a.xt = static_cast<const __nv_bfloat16*>(m.tc_xt);
  a.yt = m.tc_yt;
  a.N = m.N;
  a.K = m.K;
  a.has_base = m.has_base;
  a.n_tiles = m.tc_tiles;
  a.Q = Q;
  a.QW = ws.tc_words;
  a.ldq = ldq;
  a.C = C;
  a.active = active;
  a.P = ws.partial;
  a.NP = ws.NP;
  a.S = ws.S;
  a.err = ws.err;
  const bool xlo = m.x_dtype != GBNUTS_BF16;
  const bool split = precision == GBNUTS_PREC_BF16X3;
  dim3 grid(ws.S, (C + NCH - 1) / NCH);
  if (m.link == LINK_LOGIT) {
    if (!split) return launch_tct_t<LINK_LOGIT, false, false>(a, grid, st);
    return xlo ? launch_tct_t<LINK_LOGIT, true, true>(a, grid, st)
               : launch_tct_t<LINK_LOGIT, false, true>(a, grid, st);
  }
  if (!split) return launch_tct_t<LINK_POISSON_LOG, false, false>(a, grid, st);
  return xlo ? launch_tct_t<LINK_POISSON_LOG, true, true>(a, grid, st)
             : launch_tct_t<LINK_POISSON_LOG, false, true>(a, grid, st);
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

}  // namespace gbn

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
