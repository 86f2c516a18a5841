/*
 * trax_math.h -- project-owned FP32 math for the triplet-seeding path.
 *
 * Every transcendental the reference kernels call (OpenCL atan2, acos, atan;
 * GridBuilder.h:81, PairGeneratorBeamspot.h:138-145,212,
 * TripletThetaPhiPredictor.h:138-150,208, TripletThetaPhiFilter.h:86-99) is
 * defined here once, as __host__ __device__ code, so that the CUDA kernels and
 * the CPU oracle execute the same IEEE-754 single-precision operations in the
 * same order.  The OpenCL built-ins were vendor defined (OpenCL 1.1 allows up
 * to 6 ulp for atan2), so bit-level agreement is defined against these
 * functions, not against any particular OpenCL runtime.
 *
 * Build contract (checked by the build scripts):
 *   device: nvcc -fmad=false -prec-div=true -prec-sqrt=true -ftz=false
 *   host:   gcc/g++ -ffp-contract=off, no -ffast-math
 * With these flags every +,-,*,/ and sqrtf below is one correctly rounded
 * IEEE operation on both sides, and nothing is contracted into an FMA.
 *
 * Methods (all written for this project):
 *   trax_atan01  atan(t) for t in [0,1] as t + t^3*P(t^2), P of degree 8,
 *                coefficients fitted by fit_atan.py (Lawson-weighted least
 *                squares for minimax relative error), float32 Horner.
 *                Max error 1.1 ulp on [0,1].
 *   trax_atanf   reduction atan(x) = pi/2 - atan(1/x) for |x| > 1, odd symmetry.
 *   trax_atan2f  quadrant reduction on t = min(|x|,|y|)/max(|x|,|y|).
 *   trax_acosf   half-angle identity acos(x) = 2*atan(sqrt((1-x)/(1+x))).
 */
#ifndef TRAX_MATH_H
#define TRAX_MATH_H

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define TRAX_HD __host__ __device__ __forceinline__
#else
#define TRAX_HD static inline
#endif

/* OpenCL M_PI_F: the float nearest to pi (3.14159274f). */
#define TRAX_PI_F 0x1.921fb6p+1f
#define TRAX_TWO_PI_F 0x1.921fb6p+2f
#define TRAX_PIO2_F 0x1.921fb6p+0f
#define TRAX_3PIO4_F 0x1.2d97c8p+1f
#define TRAX_PIO4_F 0x1.921fb6p-1f

/* Grid extent (Grid.h:33-37): MIN_Z/MAX_Z = -/+300 cm, MIN/MAX_PHI = -/+ (float)M_PI. */
#define TRAX_MIN_Z (-300.0f)
#define TRAX_MAX_Z (300.0f)
#define TRAX_MIN_PHI (-TRAX_PI_F)
#define TRAX_MAX_PHI (TRAX_PI_F)

TRAX_HD float trax_atan01(float t)
{
    const float s = t * t;
    float p = -0x1.d63692p-10f;
    p = p * s; p = p + 0x1.65aaa0p-7f;
    p = p * s; p = p + -0x1.fed606p-6f;
    p = p * s; p = p + 0x1.daccb0p-5f;
    p = p * s; p = p + -0x1.583592p-4f;
    p = p * s; p = p + 0x1.c09a6ep-4f;
    p = p * s; p = p + -0x1.2421c4p-3f;
    p = p * s; p = p + 0x1.9991fep-3f;
    p = p * s; p = p + -0x1.55553ep-2f;
    float r = t * s;
    r = r * p;
    return t + r;
}

TRAX_HD float trax_atanf(float x)
{
    const float a = fabsf(x);
    if (!(a == a)) return x; /* NaN */
    float r;
    if (a > 1.0f) {
        const float inv = 1.0f / a; /* 1/inf = 0 -> pi/2 */
        r = TRAX_PIO2_F - trax_atan01(inv);
    } else {
        r = trax_atan01(a);
    }
    return copysignf(r, x);
}

/* Result lies in [-TRAX_PI_F, TRAX_PI_F]; signed zeros follow IEEE atan2. */
TRAX_HD float trax_atan2f(float y, float x)
{
    if (!(x == x) || !(y == y)) return x + y;
    const float ax = fabsf(x);
    const float ay = fabsf(y);
    float r;
    if (ay == 0.0f) {
        r = signbit(x) ? TRAX_PI_F : 0.0f;
    } else if (ax == 0.0f) {
        r = TRAX_PIO2_F;
    } else if (isinf(ax) && isinf(ay)) {
        r = signbit(x) ? TRAX_3PIO4_F : TRAX_PIO4_F;
    } else {
        const int yb = ay > ax;
        const float mx = yb ? ay : ax;
        const float mn = yb ? ax : ay;
        const float t = mn / mx;
        r = trax_atan01(t);
        if (yb) r = TRAX_PIO2_F - r;
        if (x < 0.0f) r = TRAX_PI_F - r;
    }
    return copysignf(r, y);
}

TRAX_HD float trax_acosf(float x)
{
    const float num = 1.0f - x;
    const float den = 1.0f + x;
    const float q = num / den;
    const float s = sqrtf(q);
    return 2.0f * trax_atanf(s);
}

/* OpenCL sign(): 1, -1, +/-0 for +/-0, 0 for NaN. */
TRAX_HD float trax_signf(float v)
{
    if (v > 0.0f) return 1.0f;
    if (v < 0.0f) return -1.0f;
    if (v == 0.0f) return v;
    return 0.0f;
}

/* OpenCL max()/min() on floats: "y if x < y, otherwise x" (and mirror). */
TRAX_HD float trax_maxf(float x, float y) { return (x < y) ? y : x; }
TRAX_HD float trax_minf(float x, float y) { return (y < x) ? y : x; }

/*
 * Float to integer conversions as the reference's implicit casts compile on a
 * two's-complement target: `uint u = floor(v)` truncates toward zero into a
 * 64-bit integer and keeps the low 32 bits (so -1.0f -> 0xFFFFFFFF);
 * `(int) floor(v)` saturates to INT_MIN when out of range.  NaN maps to 0 and
 * INT_MIN respectively.  Written with explicit range checks so that host and
 * device agree for every input.
 */
TRAX_HD uint32_t trax_f2u(float v)
{
    if (!(v == v)) return 0u;
    if (v >= 9.2233715e18f || v <= -9.2233715e18f) return 0u;
    if (v > -2147483648.0f && v < 2147483648.0f) return (uint32_t)(int32_t)v;
    /* |v| >= 2^31 is an integer m * 2^s (24-bit m, s >= 8): the low 32 bits
     * of its two's-complement value come from the bits, without the 64-bit
     * conversion (a slow FP64-pipe instruction on the GPU) */
    uint32_t bits;
#if defined(__CUDA_ARCH__)
    bits = __float_as_uint(v);
#else
    memcpy(&bits, &v, 4);
#endif
    const uint32_t m = (bits & 0x7FFFFFu) | 0x800000u;
    const int sh = (int)((bits >> 23) & 0xFFu) - 150;
    const uint32_t low = sh >= 32 ? 0u : m << sh;
    return (bits >> 31) ? 0u - low : low;
}

TRAX_HD int32_t trax_f2i(float v)
{
    if (!(v == v)) return INT32_MIN;
    if (v >= 2147483648.0f || v < -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}

/* Cell of a hit in its layer grid (GridBuilder.h:80-84). */
TRAX_HD uint32_t trax_sector_z(float z, float sector_size_z)
{
    return trax_f2u(floorf((z - TRAX_MIN_Z) / sector_size_z));
}

TRAX_HD uint32_t trax_sector_phi(float phi, float sector_size_phi)
{
    return trax_f2u(floorf((phi - TRAX_MIN_PHI) / sector_size_phi));
}

/*
 * floorf(x / d) for a finite d > 0, from a multiply by inv_d = 1.0f / d
 * (IEEE, computed once).  The rounded quotient RN(x / d) and q = x * inv_d
 * are both within 2^-24 (1 + 2^-24)^2 relative of the exact x / d, so they
 * differ by less than 1.5 * 2^-23 |q| as long as nothing is subnormal; when
 * q lies more than 2^-20 |q| from every integer, both have the same floor.
 * Otherwise (and for NaN, inf, |q| >= 2^22 and |q| < 2^-64) the division
 * itself is done, so the result is always floorf(x / d) bit for bit.
 */
TRAX_HD float trax_floor_div(float x, float d, float inv_d)
{
    const float q = x * inv_d;
    const float f = floorf(q);
    const float aq = fabsf(q);
    const float tol = aq * 0x1p-20f;
    if (aq < 0x1p22f && aq >= 0x1p-64f && q - f > tol && (f + 1.0f) - q > tol) return f;
    return floorf(x / d);
}

/*
 * The filter's dphi cut (TripletThetaPhiFilter.h:86-99) decided without its
 * two atan2 where the answer is certain.  The cut compares
 *   delta = wrap(trax_atan2f(dy2, dx2) - trax_atan2f(dy1, dx1))
 * with dphi.  The true angle phi from d1 = (dx1, dy1) to d2 = (dx2, dy2) is
 * atan2(cross, dot), and |delta - phi| < 3e-6: trax_atan2f is within 5e-7 of
 * atan2 (1.1 ulp polynomial on [0, 1], the division and the quadrant
 * steps), and the subtraction, the wrap by 2 * (float)pi and their roundings
 * add less than 8e-7.  cross and dot in float are each within
 * 2^-22 |d1||d2| of exact, and (cross, dot) has length |d1||d2|, so the
 * float pair's angle psi is within 4e-7 of phi.  With
 *   tlo <= tan(dphi - mu), thi >= tan(dphi + mu), mu = 2e-5
 * (each rounded outward on the host; set only for 4 mu < dphi <= 1, so that
 * 2^-24 thi stays below 1e-7):
 *   d <= 0                  |psi| >= pi/2: fails;
 *   |c| <= RN(tlo * d)      |psi| <= dphi - mu + 2^-24 tlo: passes;
 *   |c| >  RN(thi * d)      |psi| >= dphi + mu - 2^-24 thi: fails;
 * and otherwise the caller evaluates the cut itself (-1), as it does when
 * thi < 0 (screen off), for NaN or infinite input, and for vectors whose
 * 1-norm is outside [2^-40, 2^60] (no product can overflow, and underflow
 * errors stay far below 2^-22 |d1||d2|).  Returns 1 (passes), 0 (fails) or -1.
 */
#define TRAX_DPHI_SCREEN_MARGIN 2e-5
TRAX_HD int trax_dphi_screen(float dx1, float dy1, float dx2, float dy2, float tlo, float thi)
{
    const float n1 = fabsf(dx1) + fabsf(dy1), n2 = fabsf(dx2) + fabsf(dy2);
    if (!(thi >= 0.0f && n1 >= 0x1p-40f && n2 >= 0x1p-40f && n1 <= 0x1p60f && n2 <= 0x1p60f))
        return -1;
    const float c = dx1 * dy2 - dy1 * dx2;
    const float d = dx1 * dx2 + dy1 * dy2;
    if (d <= 0.0f) return 0;
    const float ac = fabsf(c);
    if (ac <= tlo * d) return 1;
    if (ac > thi * d) return 0;
    return -1;
}

/* Host side: the bounds of trax_dphi_screen for the cut dphi, from the
 * double-precision tangent rounded outward to float (thi = -1: screen off). */
static inline void trax_dphi_screen_bounds(float dphi, float *tlo, float *thi)
{
    const double mu = TRAX_DPHI_SCREEN_MARGIN;
    *tlo = -1.0f;
    *thi = -1.0f;
    if (!(dphi > 4 * mu && dphi <= 1.0f)) return;
    const double lo = tan((double)dphi - mu), hi = tan((double)dphi + mu);
    float l = (float)lo, h = (float)hi;
    if ((double)l > lo) l = nextafterf(l, 0.0f);
    if ((double)h < hi) h = nextafterf(h, 2.0f);
    *tlo = l;
    *thi = h;
}

/* GridConfig::sectorSizeZ/Phi (Grid.h:9-15), evaluated in float. */
TRAX_HD float trax_sector_size_z(uint32_t n_sectors_z)
{
    return (TRAX_MAX_Z - TRAX_MIN_Z) / (float)n_sectors_z;
}

TRAX_HD float trax_sector_size_phi(uint32_t n_sectors_phi)
{
    return (TRAX_MAX_PHI - TRAX_MIN_PHI) / (float)n_sectors_phi;
}

/* ------------------------------------------------------------------------
 * FP64 asinh for the physics evaluation's pseudorapidity
 * (PhysicsRecord.h:152-155).  The reference calls the C library's asinh; the
 * project needs one definition that host and device evaluate to the same
 * bits, so it is written here from identities:
 *   log(x):    x = m * 2^k with m in [sqrt(1/2), sqrt(2)); with
 *              s = (m - 1) / (m + 1), log(m) = 2 atanh(s) =
 *              2 (s + s^3/3 + ... + s^21/21) (|s| < 0.172, truncation
 *              below 2^-54); k ln2 with ln2 split into a 24-bit head
 *              (exact products) and a tail.
 *   log1p(y):  Goldberg's correction log(u) * y / (u - 1), u = 1 + y
 *              ("What every computer scientist should know about
 *              floating-point arithmetic", 1991, Theorem 4).
 *   asinh(t):  odd; asinh(a) = log1p(a + a^2 / (1 + sqrt(1 + a^2))) for
 *              a <= 2, log(2a + 1 / (a + sqrt(a^2 + 1))) above, log(a) + ln2
 *              beyond 2^28, a itself below 2^-28.
 * ---------------------------------------------------------------------- */
TRAX_HD uint64_t trax_d2bits(double d)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
#endif
}

TRAX_HD double trax_bits2d(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}

#define TRAX_LN2_HI 0x1.62e43p-1
#define TRAX_LN2_LO (-0x1.05c610ca86c39p-29)

/* log(x) for finite x > 0 (subnormals scaled first); NaN, 0, inf and
 * negatives follow log's special values. */
TRAX_HD double trax_log_d(double x)
{
    if (!(x == x) || x < 0.0) return trax_bits2d(0x7ff8000000000000ull);
    if (x == 0.0) return -trax_bits2d(0x7ff0000000000000ull);
    if (x == trax_bits2d(0x7ff0000000000000ull)) return x;
    int k = 0;
    if (x < 0x1p-1022) {
        x *= 0x1p54;
        k = -54;
    }
    const uint64_t u = trax_d2bits(x);
    k += (int)((u >> 52) & 0x7ff) - 1022;
    double m = trax_bits2d((u & 0x000fffffffffffffull) | 0x3fe0000000000000ull); /* [0.5, 1) */
    if (m < 0x1.6a09e667f3bcdp-1) {
        m = m * 2.0;
        k -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double p = 1.0 / 21.0;
    p = p * s2 + 1.0 / 19.0;
    p = p * s2 + 1.0 / 17.0;
    p = p * s2 + 1.0 / 15.0;
    p = p * s2 + 1.0 / 13.0;
    p = p * s2 + 1.0 / 11.0;
    p = p * s2 + 1.0 / 9.0;
    p = p * s2 + 1.0 / 7.0;
    p = p * s2 + 1.0 / 5.0;
    p = p * s2 + 1.0 / 3.0;
    const double lm = 2.0 * s + 2.0 * s * (s2 * p);
    const double kd = (double)k;
    return kd * TRAX_LN2_HI + (lm + kd * TRAX_LN2_LO);
}

TRAX_HD double trax_log1p_d(double y)
{
    const double u = 1.0 + y;
    if (u == 1.0) return y;
    return trax_log_d(u) * (y / (u - 1.0));
}

TRAX_HD double trax_asinh_d(double t)
{
    if (!(t == t)) return t;
    const double a = t < 0.0 ? -t : t;
    double r;
    if (a < 0x1p-28) {
        r = a;
    } else if (a > 0x1p28) {
        r = trax_log_d(a) + (TRAX_LN2_HI + TRAX_LN2_LO);
    } else if (a > 2.0) {
        r = trax_log_d(2.0 * a + 1.0 / (sqrt(a * a + 1.0) + a));
    } else {
        const double a2 = a * a;
        r = trax_log1p_d(a + a2 / (1.0 + sqrt(1.0 + a2)));
    }
    return t < 0.0 ? -r : r;
}

#endif /* TRAX_MATH_H */
