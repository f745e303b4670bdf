// tcgen05 / TMEM / mbarrier building blocks (inline PTX, sm_100a family).
//
// Operand tiles in shared memory use the canonical no-swizzle layouts of the
// tcgen05 matrix descriptor: 8 x 16-byte "core matrices" (8 rows of 8 bf16).
//   K-major  tile (rows r, contraction k):  off = (r/8)*SBO + (k/8)*LBO + (r%8)*16 + (k%8)*2
//            descriptor LBO = stride between core matrices along k,
//                       SBO = stride between 8-row groups.
//   MN-major tile (rows m contiguous):      off = (m/8)*SBO + (k/8)*LBO + (k%8)*16 + (m%8)*2
//            descriptor SBO = stride between 8-element m groups,
//                       LBO = stride between 8-row k groups.
// Every wait is bounded in time; on timeout the caller's error flag is set and
// the wait returns false.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace gbn {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, LBO, SBO (bytes), no swizzle,
// descriptor version 1 (bits 46-47).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: BF16 x BF16 -> FP32 (or, with f16 set,
// F16 x F16 -> FP32), dense.
__host__ __device__ constexpr uint32_t make_idesc_bf16(int M, int N, int a_mn_major,
                                                       int b_mn_major, bool f16 = false) {
  return (1u << 4)                          // D format: F32
         | ((f16 ? 0u : 1u) << 7)           // A format: BF16 (1) or F16 (0)
         | ((f16 ? 0u : 1u) << 10)          // B format: BF16 (1) or F16 (0)
         | ((uint32_t)a_mn_major << 15) | ((uint32_t)b_mn_major << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of the given parity; gives up after `limit` SM clock
// cycles, recording `code` in *err.
__device__ __forceinline__ bool mbar_wait_limit(uint64_t* bar, uint32_t parity, long long limit,
                                                int* err, int code) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) {
      if (err) atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}

// The kernels' bound: ~2 s of SM clock.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err,
                                          int code) {
  return mbar_wait_limit(bar, parity, 4000000000LL, err, code);
}

// Bounded wait that also gives up when another role has set the CTA's abort flag.
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t* bar, uint32_t parity,
                                                    volatile int* abort_flag, int* err,
                                                    int code) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort_flag) return false;
    if (clock64() - t0 > 4000000000LL) {
      *abort_flag = 1;
      if (err) atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}

// Lane 0 waits, the warp follows with the verdict (keeps .sync.aligned
// tcgen05 instructions after the wait converged).
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity,
                                          volatile int* abort_flag, int* err, int code) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) ok = mbar_wait_abortable(bar, parity, abort_flag, err, code);
  ok = __shfl_sync(0xffffffffu, ok, 0);
  __syncwarp();
  return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared (TMA engine), completing on an mbarrier.
// Addresses 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes -> visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T  (M x N x 16), issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A[tmem] * B[smem]^T (M x N x 16), A read from tensor memory
// (M lanes, 16-bit elements packed two per 32-bit column), issued by one thread.
__device__ __forceinline__ void mma_bf16_tmem_a(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc,
                                                uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// 16 consecutive 32-bit columns of this thread's TMEM lane (32x32b shape).
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}

__device__ __forceinline__ void tmem_st_wait() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Arrives on the mbarrier once every MMA this thread issued has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane (32x32b shape).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive fp32 columns of this thread's TMEM lane (32x32b shape).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 8 consecutive 32-bit columns of this thread's TMEM lane (32x32b shape).
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
      : "memory");
}

// Hardware base-2 exponential and logarithm (MUFU, approximate, flush to zero).
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Canonical K-major offset (bytes) in a tile with kt contraction elements.
__host__ __device__ __forceinline__ uint32_t kmajor_off(int r, int k, int kt) {
  return (uint32_t)((r >> 3) * (kt >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// double -> float rounded toward zero with integer operations only (the
// FP64 pipe is slow on this part): sign, rebiased exponent, top 23 mantissa
// bits; magnitudes below the float normal range give 0, above it infinity.
__device__ __forceinline__ float dbl_to_flt_rz(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
  if (e <= 0) return __int_as_float((int)sign);
  if (e >= 255) return __int_as_float((int)(sign | 0x7f800000u));
  return __int_as_float((int)(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu)));
}

// Coefficient words of the chains-on-M tensor-core kernel: theta_k and
// theta_{k+1} scaled by log2(e), split into bf16 hi and lo parts, packed two
// per 32-bit word (element k in the low half).
__device__ __forceinline__ void theta_words(double d0, double d1, uint32_t& wh, uint32_t& wl) {
  const float f0 = dbl_to_flt_rz(d0) * 1.44269504f;
  const float f1 = dbl_to_flt_rz(d1) * 1.44269504f;
  const __nv_bfloat162 hp = __floats2bfloat162_rn(f0, f1);
  const float2 hf = __bfloat1622float2(hp);
  const __nv_bfloat162 lo = __floats2bfloat162_rn(f0 - hf.x, f1 - hf.y);
  wh = *reinterpret_cast<const uint32_t*>(&hp);
  wl = *reinterpret_cast<const uint32_t*>(&lo);
}
// Words per chain: 64 hi then 64 lo (128 features), then the chain's scale
// exponent (fp16 words only) and padding to a 16-byte multiple.
constexpr int kThetaWords = 132;
constexpr int kThetaExpWord = 128;

// The fp16 form's per-chain scale: theta_k log2(e) 2^-e has its largest
// magnitude in [2^13, 2^14), so the hi parts stay far inside the fp16 range
// and the lo parts (about 2^-11 of hi) stay normal for the large components.
// fmax: largest |fp32 theta_k| log2(e) of the chain.
__host__ __device__ __forceinline__ int theta_exp_f16(float fmax) {
  if (!(fmax > 0.f) || fmax > 3.0e38f) return 0;
  int e = 0;
  frexpf(fmax, &e);  // fmax = m 2^e, m in [0.5, 1)
  e = e - 1 - 13;
  return e < -100 ? -100 : (e > 100 ? 100 : e);
}

// 2^e as a float for |e| <= 126.
__device__ __forceinline__ float exp2_int(int e) {
  return __int_as_float((127 + e) << 23);
}

// fp32 theta (already times log2(e)) pairs -> fp16 hi / lo words at scale 2^-e.
__device__ __forceinline__ void theta_words_f16(float f0, float f1, float scale, uint32_t& wh,
                                                uint32_t& wl) {
  f0 *= scale;
  f1 *= scale;
  const __half2 hp = __floats2half2_rn(f0, f1);
  const float2 hf = __half22float2(hp);
  const __half2 lo = __floats2half2_rn(f0 - hf.x, f1 - hf.y);
  wh = *reinterpret_cast<const uint32_t*>(&hp);
  wl = *reinterpret_cast<const uint32_t*>(&lo);
}

// fp32 value of a theta element as the word builders see it.
__device__ __forceinline__ float theta_f32(double d) {
  return dbl_to_flt_rz(d) * 1.44269504f;
}

// bf16 hi/lo split of a value: hi = bf16(v), lo = bf16(v - hi).
__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// fp16 hi/lo split: hi = f16(v), lo = f16(v - hi) (22 significant bits).
__device__ __forceinline__ void split_f16(float v, __half& hi, __half& lo) {
  hi = __float2half_rn(v);
  lo = __float2half_rn(v - __half2float(hi));
}

}  // namespace tc
}  // namespace gbn
