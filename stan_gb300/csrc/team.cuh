// The threads that run one chain of the sampler: one warp for small
// dimensions (four chains per CTA), or a CTA of two or four warps for large
// ones (synchronising on a named barrier).  Every thread of a team holds the chain's scalar state and executes
// the same control flow; vector work is strided over the team's threads;
// reductions combine the warps' butterfly sums in warp order (deterministic
// for a given team size).
#pragma once

namespace gbn {

struct Team {
  int t;        // thread index within the team
  int n;        // team size: 32 * nw
  int nw;       // warps in the team
  double* red;  // shared scratch, 8 doubles per warp (nw > 1)
  int bar;      // named barrier of a multi-warp team (1 or 2)

  // Barrier ids are immediates so a kernel reserves only barriers 0-2.
  __device__ __forceinline__ void sync() const {
    if (nw == 1)
      __syncwarp();
    else if (bar == 1)
      asm volatile("barrier.cta.sync 1, %0;" ::"r"(n) : "memory");
    else
      asm volatile("barrier.cta.sync 2, %0;" ::"r"(n) : "memory");
  }

  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (nw == 1) return v;
    if ((t & 31) == 0) red[(t >> 5) * 8] = v;
    sync();
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w * 8];
    sync();
    return s;
  }

  // Largest value over the team (order-independent, so deterministic).
  __device__ __forceinline__ float max(float v) const {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (nw == 1) return v;
    if ((t & 31) == 0) red[(t >> 5) * 8] = (double)v;
    sync();
    float m = v;
    for (int w = 0; w < nw; ++w) m = fmaxf(m, (float)red[w * 8]);
    sync();
    return m;
  }

  // Six sums with one pair of barriers (the U-turn dot products of a merge).
  __device__ __forceinline__ void sum6(double* v) const {
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], off);
    if (nw == 1) return;
    if ((t & 31) == 0)
#pragma unroll
      for (int j = 0; j < 6; ++j) red[(t >> 5) * 8 + j] = v[j];
    sync();
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += red[w * 8 + j];
      v[j] = s;
    }
    sync();
  }

  // f() on the team's first warp only, its value broadcast to every thread:
  // scalar FP64 work (exp, log1p) that each warp would otherwise repeat on
  // the SM's shared FP64 pipe.  Called by the whole team; slots 6 and 7 of
  // the first warp's scratch are free of the sums above.
  template <class F>
  __device__ __forceinline__ double one(F f) const {
    if (nw == 1) return f();
    double v = 0.0;
    if (t < 32) v = f();
    if (t == 0) red[7] = v;
    sync();
    v = red[7];
    sync();
    return v;
  }
  // the same for a pair of values
  template <class F>
  __device__ __forceinline__ double2 one2(F f) const {
    if (nw == 1) return f();
    double2 v = make_double2(0.0, 0.0);
    if (t < 32) v = f();
    if (t == 0) {
      red[6] = v.x;
      red[7] = v.y;
    }
    sync();
    v = make_double2(red[6], red[7]);
    sync();
    return v;
  }

  __device__ __forceinline__ bool any(bool b) const {
    if (nw == 1) return __any_sync(0xffffffffu, b) != 0;
    unsigned r;
    if (bar == 1)
      asm volatile(
          "{\n\t.reg .pred q, o;\n\t"
          "setp.ne.u32 q, %1, 0;\n\t"
          "barrier.cta.red.or.pred o, 1, %2, q;\n\t"
          "selp.u32 %0, 1, 0, o;\n\t}\n"
          : "=r"(r)
          : "r"((unsigned)b), "r"(n)
          : "memory");
    else
      asm volatile(
          "{\n\t.reg .pred q, o;\n\t"
          "setp.ne.u32 q, %1, 0;\n\t"
          "barrier.cta.red.or.pred o, 2, %2, q;\n\t"
          "selp.u32 %0, 1, 0, o;\n\t}\n"
          : "=r"(r)
          : "r"((unsigned)b), "r"(n)
          : "memory");
    return r != 0;
  }
};

}  // namespace gbn
