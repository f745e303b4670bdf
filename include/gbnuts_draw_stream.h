/*
 * gbnuts draw stream: the per-chain random-number stream consumed by the
 * NUTS sampler, defined so that the host and the GPU produce bit-identical
 * draws.
 *
 * The reference seeds one boost::random::mixmax per chain with
 * (seed, chain id) and draws uniforms and Boost normals from it
 * (src/stan/services/util/create_rng.hpp:28-34, src/stan/mcmc/hmc/base_hmc.hpp:207-210,
 * src/stan/mcmc/hmc/hamiltonians/diag_e_metric.hpp:44-50).  Neither mixmax nor
 * Boost's normal generator is reproduced here.  This stream keeps the same
 * *consumption contract* (a sequential stream of uniforms on [0,1) and a
 * sequential stream of standard normals per chain, keyed by seed and chain id)
 * with a counter-based generator, so a GPU warp can produce any element of it
 * without stepping through the ones before it.
 *
 *   generator : Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
 *               numbers: as easy as 1, 2, 3", SC'11), key = (seed, chain),
 *               counter = (block lo, block hi, stream id, 0).
 *   uniform #n: block n/2 of stream 0; words (w0,w1) for even n, (w2,w3) for
 *               odd n; value = ((w_a << 21) | (w_b >> 11)) * 2^-53  in [0,1).
 *   normal  #n: block n/2 of stream 1 gives u (from w0,w1) and v (from w2,w3);
 *               Box-Muller: r = sqrt(-2 ln(1-u)), even n -> r cos(2 pi v),
 *               odd n -> r sin(2 pi v).
 *
 * ln, sin and cos are evaluated here with explicit round-to-nearest operations
 * (series after exact argument reduction), not with the platform's libm, so
 * that the x86/Arm host build and the sm_103a build agree to the bit.
 */
#ifndef GBNUTS_DRAW_STREAM_H
#define GBNUTS_DRAW_STREAM_H

#include <stdint.h>

#if defined(__CUDACC__)
#define GBDS_FN __host__ __device__ __forceinline__
#else
#define GBDS_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define GBDS_MUL(a, b) __dmul_rn((a), (b))
#define GBDS_ADD(a, b) __dadd_rn((a), (b))
#define GBDS_SUB(a, b) __dsub_rn((a), (b))
#define GBDS_FMA(a, b, c) __fma_rn((a), (b), (c))
#define GBDS_SQRT(a) __dsqrt_rn(a)
#define GBDS_DIV(a, b) __ddiv_rn((a), (b))
#else
#include <math.h>
#include <string.h>
/* Host builds that include this header must not contract a*b+c
 * (-ffp-contract=off); the explicit forms below keep the intent visible. */
#define GBDS_MUL(a, b) ((a) * (b))
#define GBDS_ADD(a, b) ((a) + (b))
#define GBDS_SUB(a, b) ((a) - (b))
#define GBDS_FMA(a, b, c) fma((a), (b), (c))
#define GBDS_SQRT(a) sqrt(a)
#define GBDS_DIV(a, b) ((a) / (b))
#endif

#define GBDS_STREAM_UNIFORM 0u
#define GBDS_STREAM_NORMAL 1u

typedef struct {
  uint32_t w[4];
} gbds_block;

GBDS_FN uint32_t gbds_mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

/* Philox4x32 with 10 rounds. */
GBDS_FN gbds_block gbds_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                      uint32_t c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += W0;
      k1 += W1;
    }
    uint32_t hi0 = gbds_mulhi32(M0, c0), lo0 = M0 * c0;
    uint32_t hi1 = gbds_mulhi32(M1, c2), lo1 = M1 * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  gbds_block b;
  b.w[0] = c0;
  b.w[1] = c1;
  b.w[2] = c2;
  b.w[3] = c3;
  return b;
}

GBDS_FN gbds_block gbds_block_at(uint32_t seed, uint32_t chain, uint32_t stream,
                                 uint64_t block) {
  return gbds_philox4x32_10((uint32_t)block, (uint32_t)(block >> 32), stream,
                            0u, seed, chain);
}

/* Two 32-bit words -> double in [0,1) with 53 random bits. */
GBDS_FN double gbds_u01(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)a << 21) | (uint64_t)(b >> 11);
  return (double)m * 1.1102230246251565404236316680908203125e-16; /* 2^-53 */
}

GBDS_FN double gbds_uniform_at(uint32_t seed, uint32_t chain, uint64_t n) {
  gbds_block b = gbds_block_at(seed, chain, GBDS_STREAM_UNIFORM, n >> 1);
  return (n & 1u) ? gbds_u01(b.w[2], b.w[3]) : gbds_u01(b.w[0], b.w[1]);
}

GBDS_FN uint64_t gbds_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

GBDS_FN double gbds_from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

/* Natural log of a positive, normal, finite x.
 * x = m 2^e with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s), s = (m-1)/(m+1),
 * summed as s * sum_k 2 s^(2k) / (2k+1) up to k = 12 (|s| <= 0.1716, so the
 * first omitted term is below 2^-60 relative). */
GBDS_FN double gbds_ln(double x) {
  uint64_t u = gbds_bits(x);
  int e = (int)((u >> 52) & 0x7FF) - 1023;
  double m = gbds_from_bits((u & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);
  if (m > 1.4142135623730951) {
    m = GBDS_MUL(m, 0.5);
    e += 1;
  }
  double s = GBDS_DIV(GBDS_SUB(m, 1.0), GBDS_ADD(m, 1.0));
  double s2 = GBDS_MUL(s, s);
  double p = 2.0 / 25.0;
  p = GBDS_FMA(p, s2, 2.0 / 23.0);
  p = GBDS_FMA(p, s2, 2.0 / 21.0);
  p = GBDS_FMA(p, s2, 2.0 / 19.0);
  p = GBDS_FMA(p, s2, 2.0 / 17.0);
  p = GBDS_FMA(p, s2, 2.0 / 15.0);
  p = GBDS_FMA(p, s2, 2.0 / 13.0);
  p = GBDS_FMA(p, s2, 2.0 / 11.0);
  p = GBDS_FMA(p, s2, 2.0 / 9.0);
  p = GBDS_FMA(p, s2, 2.0 / 7.0);
  p = GBDS_FMA(p, s2, 2.0 / 5.0);
  p = GBDS_FMA(p, s2, 2.0 / 3.0);
  /* ln m = 2s + s*s2*p */
  double lnm = GBDS_FMA(GBDS_MUL(s, s2), p, GBDS_MUL(2.0, s));
  const double LN2_HI = 6.93147180369123816490e-01; /* high 32 bits of ln 2 */
  const double LN2_LO = 1.90821492927058770002e-10; /* ln 2 - LN2_HI */
  double de = (double)e;
  return GBDS_ADD(GBDS_MUL(de, LN2_HI), GBDS_ADD(GBDS_MUL(de, LN2_LO), lnm));
}

/* sin(x) and cos(x) for x in [0, pi/4] by their Taylor series. */
GBDS_FN void gbds_sincos_small(double x, double* s, double* c) {
  double x2 = GBDS_MUL(x, x);
  /* sin: x * (1 - x^2/3! + x^4/5! - ... - x^18/19!) */
  double ps = -1.0 / 121645100408832000.0; /* -1/19! */
  ps = GBDS_FMA(ps, x2, 1.0 / 355687428096000.0);  /* 1/17! */
  ps = GBDS_FMA(ps, x2, -1.0 / 1307674368000.0);   /* -1/15! */
  ps = GBDS_FMA(ps, x2, 1.0 / 6227020800.0);       /* 1/13! */
  ps = GBDS_FMA(ps, x2, -1.0 / 39916800.0);        /* -1/11! */
  ps = GBDS_FMA(ps, x2, 1.0 / 362880.0);           /* 1/9! */
  ps = GBDS_FMA(ps, x2, -1.0 / 5040.0);            /* -1/7! */
  ps = GBDS_FMA(ps, x2, 1.0 / 120.0);              /* 1/5! */
  ps = GBDS_FMA(ps, x2, -1.0 / 6.0);               /* -1/3! */
  *s = GBDS_FMA(GBDS_MUL(x, x2), ps, x);
  /* cos: 1 - x^2/2! + x^4/4! - ... + x^20/20! */
  double pc = 1.0 / 2432902008176640000.0;          /* 1/20! */
  pc = GBDS_FMA(pc, x2, -1.0 / 6402373705728000.0); /* -1/18! */
  pc = GBDS_FMA(pc, x2, 1.0 / 20922789888000.0);    /* 1/16! */
  pc = GBDS_FMA(pc, x2, -1.0 / 87178291200.0);      /* -1/14! */
  pc = GBDS_FMA(pc, x2, 1.0 / 479001600.0);         /* 1/12! */
  pc = GBDS_FMA(pc, x2, -1.0 / 3628800.0);          /* -1/10! */
  pc = GBDS_FMA(pc, x2, 1.0 / 40320.0);             /* 1/8! */
  pc = GBDS_FMA(pc, x2, -1.0 / 720.0);              /* -1/6! */
  pc = GBDS_FMA(pc, x2, 1.0 / 24.0);                /* 1/4! */
  pc = GBDS_FMA(pc, x2, -0.5);                      /* -1/2! */
  *c = GBDS_FMA(x2, pc, 1.0);
}

/* sin(2 pi v), cos(2 pi v) for v = k 2^-53 in [0,1): the quadrant split of 4v
 * is exact, so only the final (pi/2) * g product is rounded. */
GBDS_FN void gbds_sincos_2pi(double v, double* sn, double* cs) {
  double t = GBDS_MUL(4.0, v);
  int q = (int)t; /* 0..3 */
  double f = GBDS_SUB(t, (double)q);
  const double PIO2 = 1.57079632679489655800e+00;
  double s, c;
  if (f <= 0.5) {
    gbds_sincos_small(GBDS_MUL(PIO2, f), &s, &c);
  } else {
    double ss, cc;
    gbds_sincos_small(GBDS_MUL(PIO2, GBDS_SUB(1.0, f)), &ss, &cc);
    s = cc;
    c = ss;
  }
  switch (q) {
    case 0: *sn = s; *cs = c; break;
    case 1: *sn = c; *cs = -s; break;
    case 2: *sn = -s; *cs = -c; break;
    default: *sn = -c; *cs = s; break;
  }
}

/* Both normals of Box-Muller block b, #2b (cosine) and #2b+1 (sine), with
 * the operations of gbds_normal_at: the same two values, from one
 * logarithm and one sine/cosine evaluation. */
GBDS_FN void gbds_normal_pair_at(uint32_t seed, uint32_t chain, uint64_t block, double* z_even,
                                 double* z_odd) {
  gbds_block b = gbds_block_at(seed, chain, GBDS_STREAM_NORMAL, block);
  double u = gbds_u01(b.w[0], b.w[1]);
  double v = gbds_u01(b.w[2], b.w[3]);
  double r = GBDS_SQRT(GBDS_MUL(-2.0, gbds_ln(GBDS_SUB(1.0, u))));
  double sn, cs;
  gbds_sincos_2pi(v, &sn, &cs);
  *z_even = GBDS_MUL(r, cs);
  *z_odd = GBDS_MUL(r, sn);
}

GBDS_FN double gbds_normal_at(uint32_t seed, uint32_t chain, uint64_t n) {
  gbds_block b = gbds_block_at(seed, chain, GBDS_STREAM_NORMAL, n >> 1);
  double u = gbds_u01(b.w[0], b.w[1]);
  double v = gbds_u01(b.w[2], b.w[3]);
  double r = GBDS_SQRT(GBDS_MUL(-2.0, gbds_ln(GBDS_SUB(1.0, u))));
  double sn, cs;
  gbds_sincos_2pi(v, &sn, &cs);
  return (n & 1u) ? GBDS_MUL(r, sn) : GBDS_MUL(r, cs);
}

#endif /* GBNUTS_DRAW_STREAM_H */
