// Per-sample random streams shared by the GPU integrator and every CPU build
// that must replay the same paths.
//
// Generator: PCG32 "XSH RR" (M. E. O'Neill, "PCG: A Family of Simple Fast
// Space-Efficient Statistically Good Algorithms for Random Number Generation",
// HMC-CS-2014-0905), a 64-bit LCG with a permuted 32-bit output.  Jump-ahead
// uses F. Brown, "Random number generation with arbitrary strides" (1994).
//
// Stream layout mirrors the (seed, sequence, offset) addressing of the
// reference's curand_init(GLOBAL_SEED, pixel, frame << 32) call
// (core/random.cuh:31-39): the LCG increment is derived from the pixel's
// raster index, and sample (frame) f starts f * 2^32 draws into that stream.
// Uniforms are in (0, 1], the range curand_uniform returns.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ARR_FN __host__ __device__ __forceinline__
#else
#define ARR_FN static inline
#endif

#define AR_PCG_MULT 6364136223846793005ULL
#define AR_GLOBAL_SEED 0x9e3779b97f4a7c15ULL

struct ar_pcg
{
    uint64_t state;
    uint64_t inc;
};

// SplitMix64 finaliser (Steele, Lea & Flood 2014) to decorrelate adjacent
// pixel indices before they become LCG increments.
ARR_FN uint64_t ar_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

ARR_FN uint32_t ar_pcg_next(ar_pcg* g)
{
    const uint64_t old = g->state;
    g->state = old * AR_PCG_MULT + g->inc;
    const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
}

ARR_FN void ar_pcg_advance(ar_pcg* g, uint64_t delta)
{
    uint64_t cur_mult = AR_PCG_MULT, cur_plus = g->inc;
    uint64_t acc_mult = 1u, acc_plus = 0u;
    while (delta > 0)
    {
        if (delta & 1u)
        {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    g->state = acc_mult * g->state + acc_plus;
}

ARR_FN uint64_t ar_pcg_increment(uint64_t pixel)
{
    return (ar_mix64(pixel) << 1u) | 1u;
}

// Stream for (global seed, pixel raster index, frame / sample index).
ARR_FN ar_pcg ar_pcg_init(uint64_t seed, uint64_t pixel, uint64_t frame)
{
    ar_pcg g;
    g.state = 0u;
    g.inc = ar_pcg_increment(pixel);
    ar_pcg_next(&g);
    g.state += seed;
    ar_pcg_next(&g);
    if (frame) ar_pcg_advance(&g, frame << 32);
    return g;
}

// The jump of ar_pcg_advance is affine in the state and linear in the
// increment: advancing by delta maps state to mult * state + inc * plus1
// (mod 2^64), where mult and plus1 depend on delta alone (plus1 is the
// additive term ar_pcg_advance builds for inc = 1).  A kernel computes the
// pair once per frame and applies it per stream, with the same result as
// ar_pcg_init.
ARR_FN void ar_pcg_jump(uint64_t delta, uint64_t* mult, uint64_t* plus1)
{
    uint64_t cur_mult = AR_PCG_MULT, cur_plus = 1u;
    uint64_t acc_mult = 1u, acc_plus = 0u;
    while (delta > 0)
    {
        if (delta & 1u)
        {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    *mult = acc_mult;
    *plus1 = acc_plus;
}

// ar_pcg_init with the frame's jump given as (mult, plus1) = ar_pcg_jump(frame << 32)
ARR_FN ar_pcg ar_pcg_init_jumped(uint64_t seed, uint64_t pixel, uint64_t frame, uint64_t mult, uint64_t plus1)
{
    ar_pcg g;
    g.state = 0u;
    g.inc = ar_pcg_increment(pixel);
    ar_pcg_next(&g);
    g.state += seed;
    ar_pcg_next(&g);
    if (frame) g.state = mult * g.state + g.inc * plus1;
    return g;
}

// Uniform in (0, 1]: 24 random bits, +1, scaled exactly.
ARR_FN float ar_rand1(ar_pcg* g)
{
    return (float)((ar_pcg_next(g) >> 8) + 1u) * (1.0f / 16777216.0f);
}
