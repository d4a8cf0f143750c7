// emlab_math.h - deterministic scalar math shared by the CUDA kernels and the host setup code.
//
// The FDTD update of the reference (shaders/common.glsl:23-27, 50-54; update_E.comp:58-61;
// update_B.comp:63-64; apply_sources.comp:37-40) calls exp() for the graded-absorber profile,
// the exponential-integrator coefficients and the source footprint. GLSL leaves exp()'s accuracy
// to the GL implementation, so there is no single "right" bit pattern to reproduce. This header fixes one:
// emlab_expf is written only with IEEE operations that round identically on every conforming
// machine (multiply, add, fmaf, rintf, exponent-field construction), so the GPU kernels, the host
// coefficient tables and the CPU restatement used by the tests all get the same bits from the
// same input. Compile every user with floating-point contraction disabled (-fmad=false for nvcc,
// -ffp-contract=off for gcc) and without flush-to-zero.
//
// Method (Cody & Waite, "Software Manual for the Elementary Functions", 1980): reduce
// x = k ln2 + r with k = rint(x / ln2) and a two-part ln2 (the high part has 16 significant bits,
// so k * LN2_HI is exact for |k| <= 256), evaluate e^r on |r| <= ln2/2 with the degree-7 Taylor
// polynomial in Horner form (truncation error < 6e-9 relative, below half an ulp of float), and
// scale by 2^k through the exponent field, in two exact steps where the result is subnormal.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define EMLAB_HD __host__ __device__ __forceinline__
#else
#define EMLAB_HD static inline
#endif

#define EMLAB_LOG2E_F 1.44269502163e+00f   /* 1/ln2 rounded to float */
#define EMLAB_LN2_HI_F 6.93145751953125e-01f /* ln2 rounded to 16 significant bits */
#define EMLAB_LN2_LO_F 1.42860676533e-06f  /* ln2 - LN2_HI rounded to float */

EMLAB_HD float emlab_pow2i(int k) {
    /* 2^k as a float for k in [-126, 127]: exponent field k + 127, zero mantissa. */
    uint32_t bits = (uint32_t)(k + 127) << 23;
    float f;
    memcpy(&f, &bits, sizeof f);
    return f;
}

EMLAB_HD float emlab_expf(float x) {
    if (x != x) return x;                       /* NaN propagates */
    if (x > 88.7228394f) return INFINITY;       /* e^x above FLT_MAX */
    if (x < -103.972084f) return 0.0f;          /* e^x below half the smallest subnormal */
    const float k = rintf(x * EMLAB_LOG2E_F);
    float r = fmaf(-k, EMLAB_LN2_HI_F, x);      /* exact: k * LN2_HI has <= 24 bits */
    r = fmaf(-k, EMLAB_LN2_LO_F, r);
    float p = 1.98412701e-04f;                  /* 1/7! */
    p = fmaf(p, r, 1.38888892e-03f);            /* 1/6! */
    p = fmaf(p, r, 8.33333377e-03f);            /* 1/5! */
    p = fmaf(p, r, 4.16666679e-02f);            /* 1/4! */
    p = fmaf(p, r, 1.66666672e-01f);            /* 1/3! */
    p = fmaf(p, r, 0.5f);                       /* 1/2! */
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int ki = (int)k;
    if (ki > 127) return (p * emlab_pow2i(127)) * emlab_pow2i(ki - 127);
    if (ki < -126) return (p * emlab_pow2i(ki + 64)) * emlab_pow2i(-64);
    return p * emlab_pow2i(ki);
}

/* Absorber profile sigma(depth) = sigmaMax (e^{g u} - 1) / (e^g - 1), u = min(depth / L, 1)
   (shaders/common.glsl:23-27), in the shader's operation order. */
EMLAB_HD float emlab_pml_profile(float depth, int thickness, float sigma_max, float grading) {
    if (depth <= 0.0f) return 0.0f;
    float u = depth / (float)thickness;
    u = u < 1.0f ? u : 1.0f;
    return sigma_max * (emlab_expf(grading * u) - 1.0f) / (emlab_expf(grading) - 1.0f);
}

/* Depth of lattice coordinate c (cell units, may be a half-integer) into the absorber along one
   axis of n cells: max(L - c, c - (n - 1 - L)) (shaders/common.glsl:31-35). */
EMLAB_HD float emlab_pml_depth(float c, int n, int thickness) {
    const float L = (float)thickness;
    const float hi = (float)(n - 1) - L;
    const float a = L - c, b = c - hi;
    return a > b ? a : b;
}

/* phi(x) = (1 - e^{-x}) / x, with the 4-term series below x = 1e-2
   (shaders/common.glsl:50-54; mix(series, exact, step(1e-2, x)) selects one of the two). */
EMLAB_HD float emlab_phi(float x) {
    if (x >= 1e-2f) {
        const float d = x > 1e-12f ? x : 1e-12f;
        return (1.0f - emlab_expf(-x)) / d;
    }
    return 1.0f - x * (0.5f - x * (1.0f / 6.0f - x * (1.0f / 24.0f)));
}

/* IEEE binary16 <-> binary32 with round-to-nearest-even (the packHalf2x16 / unpackHalf2x16 pair
   the reference uses for the edge-material and thin-wire textures). */
static inline uint16_t emlab_float_to_half(float f) {
    uint32_t x;
    memcpy(&x, &f, sizeof x);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t absx = x & 0x7fffffffu;
    if (absx >= 0x7f800000u) /* inf or NaN */
        return (uint16_t)(sign | 0x7c00u | (absx > 0x7f800000u ? 0x200u : 0u));
    if (absx >= 0x477ff000u) /* rounds to >= 65520: overflow to inf */
        return (uint16_t)(sign | 0x7c00u);
    if (absx < 0x38800000u) { /* below the smallest normal half: subnormal or zero */
        if (absx < 0x33000000u) return (uint16_t)sign; /* < 2^-25 rounds to zero */
        const uint32_t e = absx >> 23;                  /* biased float exponent */
        const uint32_t m = (absx & 0x7fffffu) | 0x800000u;
        /* value / 2^-24 (the half subnormal unit) = m * 2^(e - 126): keep m >> (126 - e) */
        const uint32_t shift = 126u - e;
        uint32_t q = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u);
        const uint32_t halfway = 1u << (shift - 1u);
        if (rem > halfway || (rem == halfway && (q & 1u))) ++q;
        return (uint16_t)(sign | q);
    }
    /* normal: rebias exponent 127 -> 15, round the 13 dropped mantissa bits to nearest even */
    uint32_t h = ((absx - 0x38000000u) >> 13);
    const uint32_t rem = absx & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

static inline float emlab_half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1fu;
    const uint32_t m = h & 0x3ffu;
    uint32_t x;
    if (e == 0) {
        if (m == 0) {
            x = sign;
        } else { /* subnormal half: value m * 2^-24, exact in float */
            float f = (float)m * 5.9604644775390625e-08f;
            memcpy(&x, &f, sizeof x);
            x |= sign;
        }
    } else if (e == 31) {
        x = sign | 0x7f800000u | (m << 13);
    } else {
        x = sign | ((e + 112u) << 23) | (m << 13);
    }
    float f;
    memcpy(&f, &x, sizeof f);
    return f;
}

/* Round a float through binary16 and back: the value a shader sees after unpackHalf2x16. */
static inline float emlab_half_round(float f) { return emlab_half_to_float(emlab_float_to_half(f)); }

/* Convolutional PML (the opt-in absorber; the reference's own absorber is the graded conductivity
 * above). Coefficients of the recursive convolution of Roden & Gedney (Microwave Opt. Technol.
 * Lett. 27, 2000) with the complex-frequency-shifted stretch s = kappa + sigma / (alpha + j w):
 *   psi^{n+1} = b psi^n + c dF,   b = exp(-(sigma / kappa + alpha) dt),
 *   c = sigma / (sigma kappa + kappa^2 alpha) (b - 1),
 * and the derivative dF enters the curl as dF / kappa + psi. At coordinate u on an axis of n
 * cells with an absorber of L cells the normalised depth is delta = clamp(max(L - u, u - (n-1-L)) / L,
 * 0, 1) (the interior ends where the graded absorber's does, common.glsl:31-36), and
 *   sigma = sigma_max delta^m, kappa = 1 + (kappa_max - 1) delta^m, alpha = alpha_max (1 - delta).
 * Evaluated in FP64 on the host (library tables and the restatement alike), stored as FP32:
 * out = (b, c, 1 / kappa). */
static inline void emlab_cpml_coef(double u, int n, int L, double sigma_max, double kappa_max, double alpha_max,
                                   double order, double dt, float out[3]) {
    double d = (double)L - u, hi = u - (double)(n - 1 - L);
    if (hi > d) d = hi;
    double delta = L > 0 ? d / (double)L : 0.0;
    if (!(delta > 0.0)) delta = 0.0;
    if (delta > 1.0) delta = 1.0;
    const double g = pow(delta, order);
    const double sigma = sigma_max * g, kappa = 1.0 + (kappa_max - 1.0) * g, alpha = alpha_max * (1.0 - delta);
    const double b = exp(-(sigma / kappa + alpha) * dt);
    const double c = sigma > 0.0 ? sigma / (sigma * kappa + kappa * kappa * alpha) * (b - 1.0) : 0.0;
    out[0] = (float)b, out[1] = (float)c, out[2] = (float)(1.0 / kappa);
}
