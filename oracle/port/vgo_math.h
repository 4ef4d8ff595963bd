/* Scalar arithmetic of the CPU oracle: the reference's lane-wise math restated in plain C.
 *
 * Test infrastructure only (the CPU oracle of vamp_gb300); nothing shipped links it.
 * Compile with -ffp-contract=off: every fused multiply-add below is explicit, so the oracle
 * rounds exactly like the CUDA kernels, which emit the same operations with __fmaf_rn.
 */
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

static inline uint32_t vgo_bits(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

static inline float vgo_from_bits(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

static inline int vgo_signbit(float f)
{
    return (int)(vgo_bits(f) >> 31);
}

/* max(v, 0) and clamp(v, 0, 1) with x86 MAXPS/MINPS operand semantics (vector/avx.hh:647-656):
 * when the comparison fails (NaN, or equal zeros) the second operand is returned. */
static inline float vgo_max0(float v)
{
    return v > 0.0f ? v : 0.0f;
}

static inline float vgo_clamp01(float v)
{
    const float m = v > 0.0f ? v : 0.0f;
    return m < 1.0f ? m : 1.0f;
}

/* ---------------------------------------------------------------------------------------------
 * sin / cos.  The reference evaluates sin with the Cephes single-precision method (S. L. Moshier,
 * Cephes Math Library, sinf.c; as adapted in vector/avx.hh:456-544): reduce by multiples of pi/4
 * with an even quadrant index, a three-term Cody-Waite subtraction of pi/4, then one of two
 * minimax polynomials.  cos(x) is sin(x + pi/2) after wrapping arguments >= pi by 2 pi
 * (vector/interface.hh:451-458).  Restated with explicit fused multiply-adds. */
static inline float vgo_sin_ref(float x)
{
    uint32_t sign = vgo_bits(x) & 0x80000000u;
    const float ax = fabsf(x);
    int32_t j = (int32_t)lrintf(ax * 1.27323954473516f); /* 4 / pi, round to nearest even */
    j = (j + 1) & ~1;
    const float yj = (float)j;
    sign ^= ((uint32_t)(j & 4)) << 29;
    const int use_sin_poly = (j & 2) == 0;

    float r = fmaf(yj, -0.78515625f, ax);
    r = fmaf(yj, -2.4187564849853515625e-4f, r);
    r = fmaf(yj, -3.77489497744594108e-8f, r);
    const float z = r * r;

    float c = fmaf(2.443315711809948e-5f, z, -1.388731625493765e-3f);
    c = fmaf(c, z, 4.166664568298827e-2f);
    c = c * z;
    c = c * z;
    c = fmaf(-0.5f, z, c);
    c = c + 1.0f;

    float s = fmaf(-1.9515295891e-4f, z, 8.3321608736e-3f);
    s = fmaf(s, z, -1.6666654611e-1f);
    s = s * z;
    s = fmaf(s, r, r);

    const float y = use_sin_poly ? s : c;
    return vgo_from_bits(vgo_bits(y) ^ sign);
}

static inline float vgo_cos_ref(float x)
{
    const float pi = 3.14159265359f;
    float v = x + 1.5707963705062866f; /* (float)(pi / 2.) with pi the float above */
    if (v >= pi)
    {
        v = v - 6.2831854820251465f; /* (float)(2 * pi) */
    }
    return vgo_sin_ref(v);
}

static inline void vgo_sincos_ref(float x, float *s, float *c)
{
    *s = vgo_sin_ref(x);
    *c = vgo_cos_ref(x);
}

/* ---------------------------------------------------------------------------------------------
 * The early-exit bound of sphere_environment_in_collision (collision/validity.hh:56) computes
 * |c| with the SIMD sqrt.  On x86 that is v * RSQRTPS(v) (vector/avx.hh:412-415); the RSQRTPS
 * table measured by oracle/ref/gen_rsqrt_table.c reproduces it bit for bit.  On Arm the
 * reference uses an exact square root (vector/neon.hh:520-523). */
static const uint32_t vgo_rsqrt_x86_table[2048] = {
#include "x86_rsqrt_table.inc"
};

/* RSQRTPS(v) for v >= 2^-126 (normal, positive, finite). */
static inline float vgo_rsqrt_x86(float v)
{
    const uint32_t u = vgo_bits(v);
    const int E = (int)(u >> 23) - 127;
    const int odd = E & 1;
    const int k = (E - odd) / 2;
    const uint32_t tb = vgo_rsqrt_x86_table[((uint32_t)odd << 10) | ((u >> 13) & 1023u)];
    return vgo_from_bits((uint32_t)((int)(tb >> 23) - k) << 23 | (tb & 0x7fffffu));
}

enum
{
    VGO_SQRT_X86 = 0,  /* reference built for x86-64 (AVX2): v * rsqrt(v) */
    VGO_SQRT_EXACT = 1 /* reference built for Arm (NEON): correctly rounded sqrt */
};

/* Whether one lane of the query sphere allows the primitive loop to stop at an object with the
 * given min_distance, i.e. the sign bit of (min_distance - max_extent) is clear.
 * v = |c|^2, computed by the caller as fma(x, x, fma(z, z, y * y)). */
static inline int vgo_lane_breaks(float min_distance, float v, float r, int sqrt_mode)
{
    if (sqrt_mode == VGO_SQRT_X86)
    {
        /* zero and subnormal v: RSQRTPS returns +inf, so the bound is +inf or NaN (sign set)
         * and the lane never allows a stop */
        if (!(v >= 1.17549435e-38f))
            return 0;
        const float max_extent = fmaf(v, vgo_rsqrt_x86(v), r);
        return !vgo_signbit(min_distance - max_extent);
    }
    const float max_extent = sqrtf(v) + r;
    return !vgo_signbit(min_distance - max_extent);
}
