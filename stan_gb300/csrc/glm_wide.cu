// Batched GLM log density and gradient for wide designs (K + intercept > 128)
// on the tcgen05 tensor cores (precisions GBNUTS_PREC_BF16X3 and
// GBNUTS_PREC_BF16, logistic and Poisson), one thread-block cluster per
// (row split, group of 128 chains).
//
// The features are cut into F slabs of 128 (F = 2 or 4); CTA f of a cluster
// owns slab f: its coefficients Theta_f (bf16 hi / lo, a tensor-memory A
// operand) and its gradient accumulator G_f (tensor memory), so neither has
// to fit in one SM.  Per 128-row tile of X:
//
//   GEMM1  eta_f^T (128 chains x 128 rows) = Theta_f . X_tile,f^T   (partial eta)
//   send   the partial for the rows CTA d owns (128 / F rows each) into CTA
//          d's shared memory (distributed shared memory)
//   link   CTA f sums the F partials of its rows (in rank order, so every
//          row's eta is the same sum wherever it is computed), applies the
//          link (lp terms in a compensated fp32 sum per chain, r = d lp / d eta);
//          all 16 epilogue warps share the block, 128 / (4 F) rows each
//   share  r of its rows, as bf16 hi / lo, into every CTA's residual tile
//          (an A operand in shared memory, chains x rows, K-major)
//   GEMM2  G_f^T (128 chains x 128 feats) += R . X_tile,f             (A = R, smem)
//
// Data crossing CTAs moves with st.async, which completes its bytes on an
// mbarrier of the destination CTA; the destination arms that barrier once per
// tile with the byte count it expects and waits on it (acquire, cluster
// scope).  A sender first waits until the destination has consumed the
// previous tile's data: the destination's warps arrive remotely on the
// sender's barrier after reading their partials, and the destination's MMA
// commit (multicast to the whole cluster) marks its residual tile read.
// Every wait is bounded.
//
// X is stored per (tile, slab) as one 128 x 128 bf16 block in the canonical
// K-major core-matrix layout.  X stored in bf16 is exact; X stored in fp32 or
// fp64 is split into bf16 hi and lo parts laid out as 2 (K + intercept)
// features [hi | lo] with Theta repeated over both halves, so
// eta = (Theta_hi + Theta_lo) . (X_hi + X_lo), and the gradient of feature k
// is the sum of its hi and lo columns (written as two split partials).  Theta
// carries log2(e), so eta comes out in base-2 units for the MUFU ex2 / lg2, as
// in the narrow kernel (glm_tct.cu).
//
// TMEM (512 columns): eta partial [0, 128), G_f [128, 256), Theta_f hi
// [256, 320) and lo [320, 384).  Shared memory: a 3-stage ring of X slab
// tiles (32 KiB + y), the residual tile (hi + lo, 64 KiB), the incoming eta
// partials ((F - 1) x 128 chains x 128 / F rows fp32), lp scratch, barriers.
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
constexpr int F = 4;                    // slabs (CTAs per cluster); narrower designs pad
constexpr int RB = TM / F;              // rows of a tile whose link a CTA computes
constexpr int QR = RB / 4;              // of which each epilogue warp takes QR
constexpr int NCH = 128;                // chains per cluster (TMEM lanes)
constexpr int SLAB_BYTES = TM * TF * 2;
constexpr int STAGE_BYTES = SLAB_BYTES + 512;   // X slab tile, y (fp32 x 128)
constexpr int STAGES = 2;
constexpr int R_PART = NCH * TM * 2;    // one bf16 part of the residual tile
constexpr int R_BLOCK = NCH * RB * 2;   // one CTA's rows of one part (contiguous)
constexpr int ETA_SLOT = NCH * RB * 4;  // one source's partials for a CTA's rows
constexpr int NUM_EPI_WARPS = 16;
constexpr int THREADS = 64 + 32 * NUM_EPI_WARPS;
constexpr int SMEM_X = 0;
constexpr int SMEM_R = SMEM_X + STAGES * STAGE_BYTES;
// partials of a CTA's RB rows: a slot holds [RB / 4][NCH][4] floats (four
// rows of one chain per 16-byte chunk, chains adjacent: conflict-free 16-byte
// accesses across a warp's lanes)
constexpr int SMEM_ETA = SMEM_R + 2 * R_PART;               // incoming, F - 1 slots
constexpr int SMEM_OUT = SMEM_ETA + (F - 1) * ETA_SLOT;     // outgoing staging, F - 1 slots
constexpr int SMEM_BAR = SMEM_OUT + (F - 1) * ETA_SLOT;
constexpr int SMEM_TOTAL = SMEM_BAR + 256;
constexpr int SMEM_ALLOC = SMEM_TOTAL + 128;                // slack for 128-byte alignment
// lp scratch after the last tile ([4][NCH] + [NCH] doubles), in the outgoing
// staging buffer once every copy out of it has completed
constexpr int SMEM_LP = SMEM_OUT;
constexpr uint32_t COL_D1 = 0, COL_D2 = 128, COL_TH = 256, COL_TL = 320;
constexpr double kLn2 = 0.69314718055994530942;

// barrier slots
enum {
  B_XFULL = 0, B_XEMPTY = 2, B_D1FULL = 4, B_D1EMPTY = 5, B_THETA = 6, B_ETAIN = 7,
  B_ETAFREE = 8,   // [F]: destination d has consumed this CTA's partials
  B_RFREE = 12,    // [F]: CTA d's GEMM2 has read its residual tile
  B_RFULL = 16, B_D2FULL = 17,
  B_STAGED = 18,   // [F]: the 4 warps of sub s have staged their partials for CTA s
  B_ROWN = 22,     // the 16 epilogue warps have written this CTA's residual rows
  B_COUNT = 23
};

__device__ __forceinline__ uint64_t desc_rows(uint32_t part, int ks) {
  return make_desc(part + 256 * ks, 128, (TF / 8) * 128);
}
// The residual tile (A of GEMM2: chains x tile rows, K-major) with the rows
// outermost: element (m, k) at (k/8) 2048 + (m/8) 128 + (m%8) 16 + (k%8) 2, so
// each CTA's RB rows are one contiguous block of R_BLOCK bytes.
__device__ __forceinline__ uint32_t r_off(int m, int k) {
  return (uint32_t)((k >> 3) * 2048 + (m >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ uint64_t desc_r(uint32_t part, int ks) {
  return make_desc(part + 4096 * ks, 2048, 128);
}
__device__ __forceinline__ uint64_t desc_feats(uint32_t part, int ks) {
  return make_desc(part + 4096 * ks, (TF / 8) * 128, 128);
}

__device__ __forceinline__ uint32_t ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// The shared::cluster address of the same offset in CTA `rank`.
__device__ __forceinline__ uint32_t mapa(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
// 16 bytes into CTA-cluster shared memory; completes `bytes` on the mbarrier
// at cluster address mbar (in the same CTA as addr).
__device__ __forceinline__ void st_async_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c,
                                            uint32_t d, uint32_t mbar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];"
      ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d), "r"(mbar)
      : "memory");
}
// Bulk copy of this CTA's shared memory into CTA-cluster shared memory,
// completing `bytes` on the mbarrier at cluster address mbar (in the
// destination CTA).  Addresses 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ void bulk_copy_s2c(uint32_t dst, uint32_t src, uint32_t bytes,
                                              uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(dst), "r"(src), "r"(bytes), "r"(mbar)
      : "memory");
}
// 8 consecutive fp32 columns of this thread's TMEM lane (32x32b shape).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ double ld_cluster_f64(uint32_t addr) {
  double d;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(d) : "r"(addr) : "memory");
  return d;
}
__device__ __forceinline__ void arrive_remote(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr)
               : "memory");
}
__device__ __forceinline__ bool try_wait_cluster(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait (cluster-scope acquire) that also gives up on the CTA's abort flag.
__device__ __forceinline__ bool wait_cluster(uint64_t* bar, uint32_t parity,
                                             volatile int* abort_flag, int* err, int code) {
  const long long t0 = clock64();
  while (!try_wait_cluster(bar, parity)) {
    if (*abort_flag) return false;
    if (clock64() - t0 > 4000000000LL) {
      *abort_flag = 1;
      if (err) atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ bool warp_wait_cluster(uint64_t* bar, uint32_t parity,
                                                  volatile int* abort_flag, int* err, int code) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) ok = wait_cluster(bar, parity, abort_flag, err, code);
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}
// Arrives on the mbarrier at this offset in every CTA of ctamask once the
// MMAs this thread issued have completed.
__device__ __forceinline__ void mma_commit_multicast(uint64_t* bar, uint16_t ctamask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
      "[%0], %1;" ::"r"(smem_u32(bar)),
      "h"(ctamask)
      : "memory");
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release;" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire;" ::: "memory");
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
  constexpr uint32_t ETA_TILE = (F - 1) * ETA_SLOT;                  // partials in per tile
  constexpr uint32_t R_IN = (F - 1) * R_BLOCK * (SPLIT ? 2 : 1);    // residual bytes in per tile
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  double* sLP = reinterpret_cast<double*>(sm + SMEM_LP);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + SMEM_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + SMEM_BAR + 8 * B_COUNT);
  volatile int* abort_s = reinterpret_cast<volatile int*>(sm + SMEM_BAR + 8 * B_COUNT + 8);
  __shared__ int act_s[NCH];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = ctarank();
  const int s = blockIdx.y;
  const int c0 = blockIdx.z * NCH;

  if (tid < NCH) {
    const int cg = c0 + tid;
    act_s[tid] = (cg < a.C) && (a.active == nullptr || a.active[cg] != 0);
  }
  // every CTA of a cluster has the same chains, so a cluster leaves together
  const int any = __syncthreads_or(tid < NCH ? act_s[tid] : 0);
  if (!any) return;

  if (tid == 0) {
    for (int b = 0; b < STAGES; ++b) {
      mbar_init(&bars[B_XFULL + b], 1);
      mbar_init(&bars[B_XEMPTY + b], 1);
    }
    mbar_init(&bars[B_D1FULL], 1);
    mbar_init(&bars[B_D1EMPTY], NUM_EPI_WARPS);
    mbar_init(&bars[B_THETA], NUM_EPI_WARPS);
    // armed once per tile with the bytes the other CTAs' copies bring
    mbar_init(&bars[B_ETAIN], 1);
    // the MMA thread's arm plus this CTA's own rows
    mbar_init(&bars[B_RFULL], 2);
    for (int d = 0; d < F; ++d) {
      mbar_init(&bars[B_ETAFREE + d], NUM_EPI_WARPS);
      mbar_init(&bars[B_RFREE + d], 1);
    }
    mbar_init(&bars[B_D2FULL], 1);
    for (int d = 0; d < F; ++d) mbar_init(&bars[B_STAGED + d], 4);
    mbar_init(&bars[B_ROWN], NUM_EPI_WARPS);
    *abort_s = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, 512);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  // every CTA's barriers exist before any copy or remote arrive
  cluster_sync();
  const uint32_t tmem = *tmem_slot;

  const int t_begin = (int)((long long)a.n_tiles * s / a.S);
  const int t_end = (int)((long long)a.n_tiles * (s + 1) / a.S);
  const int n = t_end - t_begin;
  const uint32_t sm_base = smem_u32(sm);

  if (warp == 0) {
    // ---- producer: this CTA's slab of each tile through the ring
    if (lane == 0) {
      for (int i = 0; i < n; ++i) {
        const int st = i % STAGES, u = i / STAGES;
        if (!mbar_wait_abortable(&bars[B_XEMPTY + st], (u & 1) ^ 1, abort_s, a.err, 41)) break;
        unsigned char* dst = sm + SMEM_X + st * STAGE_BYTES;
        const uint16_t* src = a.xt + ((size_t)(t_begin + i) * F + rank) * (TM * TF);
        mbar_arrive_expect_tx(&bars[B_XFULL + st], SLAB_BYTES + TM * 4);
        bulk_copy_g2s(dst, src, SLAB_BYTES, &bars[B_XFULL + st]);
        bulk_copy_g2s(dst + SLAB_BYTES, a.yt + (size_t)(t_begin + i) * TM, TM * 4,
                      &bars[B_XFULL + st]);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---- MMA issuer: GEMM1 of tile i, then GEMM2 of tile i - 1
    if (lane == 0) {
      const uint32_t id1 = make_idesc_bf16(NCH, TM, 0, 0);
      const uint32_t id2 = make_idesc_bf16(NCH, TF, 0, 1);
      const uint32_t rh = sm_base + SMEM_R, rl = rh + R_PART;
      const uint16_t all = (uint16_t)((1u << F) - 1);
      if (n > 0) mbar_arrive_expect_tx(&bars[B_RFULL], R_IN);
      bool ok = mbar_wait_abortable(&bars[B_THETA], 0, abort_s, a.err, 42);
      fence_after_sync();
      auto gemm2 = [&](int i) -> bool {
        if (!wait_cluster(&bars[B_RFULL], i & 1, abort_s, a.err, 43)) return false;
        fence_after_sync();
        const int st = i % STAGES;
        const uint32_t xs = sm_base + SMEM_X + st * STAGE_BYTES;
#pragma unroll 1
        for (int ks = 0; ks < TM / 16; ++ks) {
          const uint64_t bx = desc_feats(xs, ks);
          mma_bf16(tmem + COL_D2, desc_r(rh, ks), bx, id2, (i > 0 || ks > 0) ? 1u : 0u);
          if (SPLIT) mma_bf16(tmem + COL_D2, desc_r(rl, ks), bx, id2, 1u);
        }
        mma_commit_multicast(&bars[B_RFREE + rank], all);
        mma_commit(&bars[B_XEMPTY + st]);
        if (i + 1 < n) mbar_arrive_expect_tx(&bars[B_RFULL], R_IN);
        return true;
      };
      for (int i = 0; i < n && ok; ++i) {
        const int st = i % STAGES;
        ok = mbar_wait_abortable(&bars[B_XFULL + st], (i / STAGES) & 1, abort_s, a.err, 44) &&
             mbar_wait_abortable(&bars[B_D1EMPTY], (i & 1) ^ 1, abort_s, a.err, 45);
        if (!ok) break;
        fence_after_sync();
        const uint32_t xs = sm_base + SMEM_X + st * STAGE_BYTES;
#pragma unroll 1
        for (int ks = 0; ks < TF / 16; ++ks) {
          const uint64_t bx = desc_rows(xs, ks);
          mma_bf16_tmem_a(tmem + COL_D1, tmem + COL_TH + 8 * ks, bx, id1, ks > 0 ? 1u : 0u);
          if (SPLIT) mma_bf16_tmem_a(tmem + COL_D1, tmem + COL_TL + 8 * ks, bx, id1, 1u);
        }
        mma_commit(&bars[B_D1FULL]);
        if (i > 0) ok = gemm2(i - 1);
      }
      if (ok && n > 0) ok = gemm2(n - 1);
      mma_commit(&bars[B_D2FULL]);
      mbar_wait(&bars[B_D2FULL], 0, a.err, 49);
    }
    __syncwarp();
  } else {
    // ---- epilogue: warp (q, sub) owns chains 32q.. (TMEM lane quarter q).
    // Sub s's eta partial columns 32 s .. are the rows of CTA s: staged and
    // bulk-copied there (sub == rank: this CTA's own rows).  Every warp then
    // computes the link of QR of this CTA's own rows.
    const int q = warp & 3;
    const int sub = (warp - 2) >> 2;
    const int c = 32 * q + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
    const int own0 = RB * (int)rank + QR * sub;   // first own row (tile row index)
    const int oslot = sub < (int)rank ? sub : sub - 1;       // outgoing staging slot
    const int islot = (int)rank < sub ? (int)rank : (int)rank - 1;  // my slot at CTA sub
    {
      // log2(e) Theta_f of this chain -> TMEM (features 32 sub .. of the slab)
      const bool act = act_s[c] != 0;
      const double* th = a.Q + (size_t)(act ? c0 + c : 0) * a.ldq;
      uint32_t wh[16], wl[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        double d2[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int fj = (int)rank * TF + 32 * sub + 2 * j + e;  // feature of the layout
          const int k = fj < a.kx ? fj : (a.doubled && fj < 2 * a.kx ? fj - a.kx : -1);
          d2[e] = (act && k >= 0) ? th[k] : 0.0;
        }
        theta_words(d2[0], d2[1], wh[j], wl[j]);
      }
      tmem_st16(lane_addr + COL_TH + 16 * sub, wh);
      tmem_st16(lane_addr + COL_TL + 16 * sub, wl);
      tmem_st_wait();
      fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars[B_THETA]);
    }
    float2 sa = make_float2(0.f, 0.f), sb = make_float2(0.f, 0.f);
    bool ok = true;
    for (int i = 0; i < n && ok; ++i) {
      const int st = i % STAGES;
      if (warp == 2 && lane == 0) mbar_arrive_expect_tx(&bars[B_ETAIN], ETA_TILE);
      if (!warp_wait(&bars[B_D1FULL], i & 1, abort_s, a.err, 46)) {
        ok = false;
        break;
      }
      fence_after_sync();
      float v[32], o[QR];
      tmem_ld32(lane_addr + COL_D1 + 32 * sub, v);
      tmem_ld8(lane_addr + COL_D1 + own0, o);
      tmem_ld_wait();
      fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars[B_D1EMPTY]);
      if (sub != (int)rank) {
        // stage the partial for CTA sub's rows (the staging slot is free once
        // CTA sub has consumed the previous tile), then one bulk copy
        if (!warp_wait_cluster(&bars[B_ETAFREE + sub], (i & 1) ^ 1, abort_s, a.err, 47)) {
          ok = false;
          break;
        }
        float4* stg = reinterpret_cast<float4*>(sm + SMEM_OUT + oslot * ETA_SLOT) + c;
#pragma unroll
        for (int j = 0; j < 32; j += 4)
          stg[(j >> 2) * NCH] = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_arrive(&bars[B_STAGED + sub]);
        if (q == 0 && lane == 0) {
          ok = mbar_wait_abortable(&bars[B_STAGED + sub], i & 1, abort_s, a.err, 52);
          if (ok)
            bulk_copy_s2c(mapa(sm_base + SMEM_ETA + (uint32_t)(islot * ETA_SLOT), (uint32_t)sub),
                          sm_base + SMEM_OUT + (uint32_t)(oslot * ETA_SLOT), ETA_SLOT,
                          mapa(smem_u32(&bars[B_ETAIN]), (uint32_t)sub));
        }
        ok = __shfl_sync(0xffffffffu, (int)ok, 0) != 0;
        if (!ok) break;
      }
      // ---- own rows: the F partials summed in rank order, then the link
      if (!warp_wait_cluster(&bars[B_ETAIN], i & 1, abort_s, a.err, 48)) {
        ok = false;
        break;
      }
      float e2[QR];
#pragma unroll
      for (int j = 0; j < QR; ++j) e2[j] = 0.f;
#pragma unroll
      for (int r = 0; r < F; ++r) {
        if (r == (int)rank) {
#pragma unroll
          for (int j = 0; j < QR; ++j) e2[j] += o[j];
        } else {
          const int slot = r < (int)rank ? r : r - 1;
          const float4* src = reinterpret_cast<const float4*>(sm + SMEM_ETA + slot * ETA_SLOT) +
                              (QR * sub / 4) * NCH + c;
#pragma unroll
          for (int j = 0; j < QR; j += 4) {
            const float4 p = src[(j >> 2) * NCH];
            e2[j] += p.x;
            e2[j + 1] += p.y;
            e2[j + 2] += p.z;
            e2[j + 3] += p.w;
          }
        }
      }
      __syncwarp();
      if (lane < F && lane != (int)rank)
        arrive_remote(mapa(smem_u32(&bars[B_ETAFREE + rank]), (uint32_t)lane));
      const float* ys =
          reinterpret_cast<const float*>(sm + SMEM_X + st * STAGE_BYTES + SLAB_BYTES) + own0;
      const long long row0 = (long long)(t_begin + i) * TM + own0;
      const int nvalid = (int)max(0LL, min((long long)QR, a.N - row0));
      float pa = 0.f, pb = 0.f;
      uint32_t wh[QR / 2], wl[QR / 2];
#pragma unroll
      for (int j = 0; j < QR; j += 2) {
        float res[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const float x = e2[j + e];
          const float yv = ys[j + e];
          float ta, tb = 0.f, r;
          if (LINK == LINK_LOGIT) {
            const float ex = ex2_approx(-fabsf(x));
            const float dd = 1.f + ex;
            const float inv = rcp_approx(dd);
            const float sig = x >= 0.f ? inv : ex * inv;
            ta = yv * x - fmaxf(x, 0.f) - lg2_approx(dd);
            r = yv - sig;
          } else {
            const float mu = ex2_approx(x);
            ta = yv * x;
            tb = mu;
            r = yv - mu;
          }
          if (j + e >= nvalid) {
            ta = 0.f;
            tb = 0.f;
            r = 0.f;
          }
          pa += ta;
          pb += tb;
          res[e] = r;
        }
        const __nv_bfloat162 hp = __floats2bfloat162_rn(res[0], res[1]);
        const float2 hf = __bfloat1622float2(hp);
        const __nv_bfloat162 lo = __floats2bfloat162_rn(res[0] - hf.x, res[1] - hf.y);
        wh[j >> 1] = *reinterpret_cast<const uint32_t*>(&hp);
        wl[j >> 1] = *reinterpret_cast<const uint32_t*>(&lo);
      }
      two_sum_add(sa, pa);
      if (LINK != LINK_LOGIT) two_sum_add(sb, pb);
      // ---- residual rows own0 .. of chain c into this CTA's residual tile,
      // once every CTA's GEMM2 of the previous tile is done (they read this
      // CTA's block through the copies below); then one thread copies the
      // block to the other CTAs
      if (lane == 0)
        for (int d = 0; d < F && ok; ++d)
          ok = wait_cluster(&bars[B_RFREE + d], (i & 1) ^ 1, abort_s, a.err, 50);
      ok = __shfl_sync(0xffffffffu, (int)ok, 0) != 0;
      if (!ok) break;
      const uint32_t off = r_off(c, own0);
      *reinterpret_cast<uint4*>(sm + SMEM_R + off) = make_uint4(wh[0], wh[1], wh[2], wh[3]);
      if (SPLIT)
        *reinterpret_cast<uint4*>(sm + SMEM_R + R_PART + off) =
            make_uint4(wl[0], wl[1], wl[2], wl[3]);
      fence_proxy_async();
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars[B_ROWN]);
      if (warp == 2 && lane == 0) {
        ok = mbar_wait_abortable(&bars[B_ROWN], i & 1, abort_s, a.err, 53);
        if (ok) {
          mbar_arrive(&bars[B_RFULL]);
          const uint32_t blk = (uint32_t)(rank * R_BLOCK);
          for (int d = 0; d < F; ++d) {
            if (d == (int)rank) continue;
            const uint32_t rbar = mapa(smem_u32(&bars[B_RFULL]), (uint32_t)d);
            const uint32_t dst = mapa(sm_base + SMEM_R, (uint32_t)d);
            bulk_copy_s2c(dst + blk, sm_base + SMEM_R + blk, R_BLOCK, rbar);
            if (SPLIT)
              bulk_copy_s2c(dst + R_PART + blk, sm_base + SMEM_R + R_PART + blk, R_BLOCK, rbar);
          }
        }
      }
      ok = __shfl_sync(0xffffffffu, (int)ok, 0) != 0;
    }
    // per-chain lp of this warp's rows, in the staging buffer once every
    // copy out of it has completed (each destination has consumed the last
    // tile's partials)
    if (lane == 0 && n > 0)
      for (int d = 0; d < F; ++d)
        if (d != (int)rank) wait_cluster(&bars[B_ETAFREE + d], (n - 1) & 1, abort_s, a.err, 54);
    __syncwarp();
    sLP[sub * NCH + c] = kLn2 * ((double)sa.x + (double)sa.y) - ((double)sb.x + (double)sb.y);
    // gradient partials: features 32 sub .. of the slab
    if (ok && warp_wait(&bars[B_D2FULL], 0, abort_s, a.err, 51)) {
      fence_after_sync();
      float g[32];
      tmem_ld32(lane_addr + COL_D2 + 32 * sub, g);
      tmem_ld_wait();
      if (act_s[c]) {
        for (int j = 0; j < 32; ++j) {
          const int fj = (int)rank * TF + 32 * sub + j;
          int k = fj, part = 0;
          if (fj >= a.kx) {
            if (!a.doubled || fj >= 2 * a.kx) continue;
            k = fj - a.kx;
            part = 1;
          }
          double* dst = a.P + ((size_t)(part * a.S + s) * a.C + c0 + c) * a.NP;
          if (k < a.has_base)
            dst[1] = (double)g[j];
          else
            dst[4 + (k - a.has_base)] = (double)g[j];
        }
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  // this CTA's lp per chain, then the cluster's total (rank 0, rank order)
  double* sTot = sLP + 4 * NCH;
  if (tid < NCH) {
    double t = 0.0;
    for (int k = 0; k < 4; ++k) t += sLP[k * NCH + tid];
    sTot[tid] = t;
  }
  cluster_sync();
  if (rank == 0 && tid < NCH && act_s[tid]) {
    double lp = 0.0;
    for (int r = 0; r < F; ++r) lp += ld_cluster_f64(mapa(smem_u32(&sTot[tid]), (uint32_t)r));
    double* dst = a.P + ((size_t)s * a.C + c0 + tid) * a.NP;
    dst[0] = lp;
    dst[2] = 0.0;
    dst[3] = 0.0;
    if (a.doubled) {
      double* d2 = a.P + ((size_t)(a.S + s) * a.C + c0 + tid) * a.NP;
      d2[0] = 0.0;
      d2[2] = 0.0;
      d2[3] = 0.0;
    }
  }
  // no CTA leaves while another may still read its shared memory
  cluster_sync();
  if (warp == 0) {
    fence_after_sync();
    tmem_dealloc(tmem, 512);
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

namespace {
// Clusters of F CTAs that fit on the device at once (one CTA per SM).
int max_clusters() {
  int dev = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<int, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  const void* k = reinterpret_cast<const void*>(glm_wide_kernel<LINK_LOGIT, true>);
  int n = 0;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, wide::SMEM_ALLOC) ==
      cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(wide::F, 1, 1);
    cfg.blockDim = dim3(wide::THREADS, 1, 1);
    cfg.dynamicSmemBytes = wide::SMEM_ALLOC;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = wide::F;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) n = 0;
  }
  cudaGetLastError();
  if (n <= 0) n = std::max(1, device_sm_count() / wide::F);
  cache[dev] = n;
  return n;
}
}  // namespace

int wide_splits(const ModelDesc& m, int C) {
  const int F = wide_slabs(m);
  if (F == 0) return 1;
  const int groups = (C + wide::NCH - 1) / wide::NCH;
  const int tiles = (int)((m.N + wide::TM - 1) / wide::TM);
  int S = std::max(1, max_clusters() / groups);
  S = std::min(S, std::max(1, tiles));
  return S;
}

template <int LINK, bool SPLIT>
static int launch_wide_t(const WideArgs& a, int groups, cudaStream_t st) {
  using namespace wide;
  int rc = ensure_smem(glm_wide_kernel<LINK, SPLIT>, SMEM_ALLOC);
  if (rc) return rc;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(F, a.S, groups);
  cfg.blockDim = dim3(THREADS, 1, 1);
  cfg.dynamicSmemBytes = SMEM_ALLOC;
  cfg.stream = st;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = F;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  GBN_CUDA_TRY(cudaLaunchKernelEx(&cfg, glm_wide_kernel<LINK, SPLIT>, a));
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
  const int groups = (C + wide::NCH - 1) / wide::NCH;
  const bool split = precision == GBNUTS_PREC_BF16X3;
  if (m.link == LINK_LOGIT)
    return split ? launch_wide_t<LINK_LOGIT, true>(a, groups, st)
                 : launch_wide_t<LINK_LOGIT, false>(a, groups, st);
  return split ? launch_wide_t<LINK_POISSON_LOG, true>(a, groups, st)
               : launch_wide_t<LINK_POISSON_LOG, false>(a, groups, st);
}

}  // namespace gbn

