// The threads that run one chain of the sampler: one warp (four chains per
// CTA) for small dimensions, or a whole CTA of two or four warps for large
// ones.  Every thread of a team holds the chain's scalar state and executes
// the same control flow; vector work is strided over the team's threads;
// reductions combine the warps' butterfly sums in warp order (deterministic
// for a given team size).
#pragma once

namespace gbn {

struct Team {
  int t;        // thread index within the team
  int n;        // team size: 32 * nw
  int nw;       // warps in the team (1, or the whole CTA)
  double* red;  // shared scratch, 8 doubles per warp (nw > 1)

  __device__ __forceinline__ void sync() const {
    if (nw == 1)
      __syncwarp();
    else
      __syncthreads();
  }

  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (nw == 1) return v;
    if ((t & 31) == 0) red[(t >> 5) * 8] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w * 8];
    __syncthreads();
    return s;
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
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += red[w * 8 + j];
      v[j] = s;
    }
    __syncthreads();
  }

  __device__ __forceinline__ bool any(bool b) const {
    if (nw == 1) return __any_sync(0xffffffffu, b) != 0;
    return __syncthreads_or(b) != 0;
  }
};

}  // namespace gbn
