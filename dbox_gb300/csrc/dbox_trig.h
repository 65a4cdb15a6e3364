// Portable float sine/cosine used by every rotation update of the step
// (b2Rot.Set in common/b2math.d:478-488; called from b2Body.SynchronizeTransform
// b2body.d:1143-1147, b2Sweep.GetTransform b2math.d:556-564 and the position
// solvers b2contactsolver.d:96-100).
//
// The reference calls the C runtime's sinf/cosf, whose results are not
// correctly rounded (glibc 2.39 differs from the correctly rounded value on
// about 1% of inputs) and whose algorithm is not part of this project.  This
// header has its own evaluation, written only with IEEE binary32/binary64
// +, -, *, / and explicit correctly rounded fused multiply-add (fmaf on the
// host, __fmaf_rn on the device).  Compilers may not contract anything else
// (gcc -ffp-contract=off, nvcc --fmad=false), so the host and the device
// produce identical bits for every input.
//
// Method (published methods, restated here):
//  * |x| <= 1024, binary32: Cody & Waite additive reduction by pi/2 with pi/2
//    split into 13 + 13 + 24 + 24 bits (k*A and k*B are exact for |k| < 2^10),
//    the reduced argument kept as an unevaluated float pair (Knuth's TwoSum and
//    the FMA product error); Taylor polynomials of sin and cos in Horner form
//    with the leading terms summed in float pairs.  Error below 0.6 ulp over the
//    whole range (measured exhaustively against the correctly rounded value).
//  * |x| > 1024, binary64: Cody & Waite with a 33 + 33 + 53-bit split below 2^17,
//    Payne & Hanek reduction above (24-bit chunks of 2/pi, double-double sum),
//    Taylor polynomials through r^21 / r^20, rounded once to binary32.
#pragma once

#ifdef __CUDACC__
#define DBOX_TRIG_HD __host__ __device__ __forceinline__
#else
#define DBOX_TRIG_HD static inline
#endif

#include <stdint.h>
#include <math.h>

namespace dbox_trig {

DBOX_TRIG_HD float fma_f(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

// Knuth TwoSum: s + e == a + b exactly
DBOX_TRIG_HD void two_sum_f(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Bits of 2/pi after the binary point, 24 per entry (mpmath, 2000-bit precision).
#ifdef __CUDACC__
__host__ __device__
#endif
static inline uint32_t two_over_pi_chunk(int i) {
    // A switch keeps the table out of host/device global memory declarations.
    switch (i) {
    case 0: return 0xA2F983u; case 1: return 0x6E4E44u; case 2: return 0x1529FCu;
    case 3: return 0x2757D1u; case 4: return 0xF534DDu; case 5: return 0xC0DB62u;
    case 6: return 0x95993Cu; case 7: return 0x439041u; case 8: return 0xFE5163u;
    case 9: return 0xABDEBBu; case 10: return 0xC561B7u; default: return 0x246E3Au;
    }
}

DBOX_TRIG_HD double ldexp_i(double v, int e) {
    // exact scaling by 2^e for |e| <= 1000 via repeated exact multiplies
    while (e > 60) { v *= 0x1p60; e -= 60; }      // 2^60
    while (e < -60) { v *= 0x1p-60; e += 60; }      // 2^-60
    uint64_t bits = (uint64_t)(e + 1023) << 52;
    double s;
    // type pun through a union-free memcpy equivalent
    union { uint64_t u; double d; } cv; cv.u = bits; s = cv.d;
    return v * s;
}

DBOX_TRIG_HD void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Reduce |x| (as a float) to r in about [-pi/4, pi/4] and quadrant q in 0..3.
DBOX_TRIG_HD void reduce(float ax, double& r, int& q) {
    const double INV_PIO2 = 0x1.45f306dc9c883p-1;
    const double P1 = 0x1.921fb54400000p+0;
    const double P2 = 0x1.0b4611a600000p-34;
    const double P3 = 0x1.3198a2e037073p-69;
    const double PIO2 = 0x1.921fb54442d18p+0;
    const double MAGIC = 6755399441055744.0;  // 1.5 * 2^52: round to nearest integer
    double xd = (double)ax;
    if (ax < 131072.0f) {
        double t = xd * INV_PIO2;
        t = t + MAGIC;
        t = t - MAGIC;
        r = ((xd - t * P1) - t * P2) - t * P3;
        q = ((int)t) & 3;
        return;
    }
    // Payne-Hanek for large arguments: ax = m * 2^e2 with 2^23 <= m < 2^24.
    union { float f; uint32_t u; } cv; cv.f = ax;
    int bexp = (int)((cv.u >> 23) & 0xff);
    uint32_t m = (cv.u & 0x7fffffu) | 0x800000u;
    int e2 = bexp - 127 - 23;
    int i0 = (e2 - 2) / 24;  // e2 >= -6 here so e2-2 >= -8; C division truncates toward 0
    if (e2 - 2 < 0) i0 = 0;
    double hi = 0.0, lo = 0.0;
    for (int i = i0; i < i0 + 6; ++i) {
        double term = ldexp_i((double)((uint64_t)m * (uint64_t)two_over_pi_chunk(i)), e2 - 24 * (i + 1));
        if (i == i0) {
            // drop whole multiples of 4 (they do not change sin/cos)
            double q4 = term * 0.25;
            q4 = q4 + MAGIC; q4 = q4 - MAGIC;   // nearest integer of term/4
            if (q4 * 4.0 > term) q4 -= 1.0;     // make it floor
            term = term - q4 * 4.0;             // exact: both are multiples of the term's ulp
            hi = term;
        } else {
            double s, e;
            two_sum(hi, term, s, e);
            hi = s;
            lo += e;
        }
    }
    double k = hi + MAGIC; k = k - MAGIC;       // nearest integer to hi
    double f = (hi - k) + lo;
    r = f * PIO2;
    q = ((int)k) & 3;
}

DBOX_TRIG_HD double sin_poly(double r) {
    const double r2 = r * r;
    double p = 0x1.71b8ef6dcf572p-66;            //  1/21!
    p = -0x1.2f49b46814157p-57 + r2 * p;         // -1/19!
    p =  0x1.952c77030ad4ap-49 + r2 * p;         //  1/17!
    p = -0x1.ae7f3e733b81fp-41 + r2 * p;         // -1/15!
    p =  0x1.6124613a86d09p-33 + r2 * p;         //  1/13!
    p = -0x1.ae64567f544e4p-26 + r2 * p;         // -1/11!
    p =  0x1.71de3a556c734p-19 + r2 * p;         //  1/9!
    p = -0x1.a01a01a01a01ap-13 + r2 * p;         // -1/7!
    p =  0x1.1111111111111p-7 + r2 * p;          //  1/5!
    p = -0x1.5555555555555p-3 + r2 * p;          // -1/3!
    return r + (r * r2) * p;
}

DBOX_TRIG_HD double cos_poly(double r) {
    const double r2 = r * r;
    double p = 0x1.e542ba4020225p-62;            //  1/20!
    p = -0x1.6827863b97d97p-53 + r2 * p;         // -1/18!
    p =  0x1.ae7f3e733b81fp-45 + r2 * p;         //  1/16!
    p = -0x1.93974a8c07c9dp-37 + r2 * p;         // -1/14!
    p =  0x1.1eed8eff8d898p-29 + r2 * p;         //  1/12!
    p = -0x1.27e4fb7789f5cp-22 + r2 * p;         // -1/10!
    p =  0x1.a01a01a01a01ap-16 + r2 * p;         //  1/8!
    p = -0x1.6c16c16c16c17p-10 + r2 * p;         // -1/6!
    p =  0x1.5555555555555p-5 + r2 * p;          //  1/4!
    p = -0x1.0000000000000p-1 + r2 * p;          // -1/2!
    return 1.0 + r2 * p;
}

// sin and cos of a binary32 angle through binary64 (used above |x| = 1024).
DBOX_TRIG_HD void sincos_f64(float x, float* s_out, float* c_out) {
    float ax = x < 0.0f ? -x : x;
    double r; int q;
    reduce(ax, r, q);
    double sr = sin_poly(r);
    double cr = cos_poly(r);
    double s, c;
    switch (q) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
    }
    if (x < 0.0f) s = -s;
    *s_out = (float)s;
    *c_out = (float)c;
}

// sin and cos of a binary32 angle with |x| <= 1024, in binary32 with FMA.
DBOX_TRIG_HD void sincos_f32(float x, float* s_out, float* c_out) {
    const float INV_PIO2 = 0x1.45f306p-1f;
    const float MAGIC = 12582912.0f;                 // 1.5 * 2^23: round to nearest integer
    const float A = 0x1.921p+0f;                     // pi/2 = A + B + C + D
    const float B = 0x1.f6ap-13f;
    const float C = 0x1.110b46p-26f;
    const float D = 0x1.1a6264p-54f;
    float k = (x * INV_PIO2 + MAGIC) - MAGIC;
    float r1 = fma_f(-k, A, x);                      // exact
    float rh, rl;
    two_sum_f(r1, -(k * B), rh, rl);                 // k*B exact
    float p3 = k * C;
    float e3 = fma_f(k, C, -p3);                     // k*C == p3 + e3
    float t, e;
    two_sum_f(rh, -p3, t, e);
    float small = ((rl + e) - e3) - k * D;
    two_sum_f(t, small, rh, rl);                     // reduced argument r = rh + rl
    float z = rh * rh;
    float ez = fma_f(rh, rh, -z);                    // rh^2 == z + ez
    // sin r = r + r^3 (-1/6 + r^2/120 - r^4/5040 + r^6/362880) + ...
    float ps = fma_f(z, fma_f(z, fma_f(z, 0x1.71de3ap-19f, -0x1.a01a02p-13f), 0x1.111112p-7f), -0x1.555556p-3f);
    float sin_lo = fma_f(rh * z, ps, rl - 0.5f * z * rl);
    float sr = rh + sin_lo;
    // cos r = 1 - r^2/2 + r^4 (1/24 - r^2/720 + r^4/40320 - r^6/3628800 + r^8/479001600) + ...
    float pc = fma_f(z, fma_f(z, fma_f(z, fma_f(z, 0x1.1eed8ep-29f, -0x1.27e4fcp-22f), 0x1.a01a02p-16f),
                              -0x1.6c16c2p-10f), 0x1.555556p-5f);
    float w = 0.5f * z;
    float hi = 1.0f - w;
    float lo = (1.0f - hi) - w;                      // exact: |w| <= 0.31
    float cos_lo = ((lo - 0.5f * ez) - rh * rl) + (z * z) * pc;
    float cr = hi + cos_lo;
    // quadrant q: (sin, cos) = (sr, cr), (cr, -sr), (-sr, -cr), (-cr, sr) for q = 0..3
    int q = ((int)k) & 3;
    float s = (q & 1) ? cr : sr;
    float c = (q & 1) ? sr : cr;
    if (q & 2) s = -s;
    if ((q + 1) & 2) c = -c;
    *s_out = s;
    *c_out = c;
}

#ifdef __CUDACC__
// the binary64 path as one out-of-line device function: it runs for |x| > 1024 only, and a
// copy inlined at every rotation would fill the instruction cache with code that never runs
static __device__ __noinline__ void sincos_f64_cold(float x, float* s_out, float* c_out) { sincos_f64(x, s_out, c_out); }
#endif

}  // namespace dbox_trig

// sin and cos of a binary32 angle (b2Rot.Set): identical bits on the host and the device.
DBOX_TRIG_HD void dbox_sincosf(float x, float* s_out, float* c_out) {
#ifdef __CUDA_ARCH__
    // device: the binary32 path runs for every input and the rare cases are patched after
    // it, so the lanes of a warp stay on one path (same results as the branches below)
    float s, c;
    dbox_trig::sincos_f32(x, &s, &c);
    float ax = fabsf(x);
    if (!(ax <= 1024.0f)) {
        if (ax == ax && ax != __int_as_float(0x7f800000)) {
            dbox_trig::sincos_f64_cold(x, &s, &c);
        } else {
            s = x - x;
            c = s;
        }
    }
    if (x == 0.0f) { s = x; c = 1.0f; }
    *s_out = s;
    *c_out = c;
#else
    union { float f; uint32_t u; } cv; cv.f = x;
    if ((cv.u & 0x7f800000u) == 0x7f800000u) {  // inf or nan
        float n = x - x;
        *s_out = n; *c_out = n;
        return;
    }
    if (x == 0.0f) { *s_out = x; *c_out = 1.0f; return; }   // sin(-0) = -0
    float ax = x < 0.0f ? -x : x;
    if (ax <= 1024.0f) dbox_trig::sincos_f32(x, s_out, c_out);
    else dbox_trig::sincos_f64(x, s_out, c_out);
#endif
}
