// sinf / cosf that return, bit for bit, what the host C library returns: the zeroth-phase call of the MESE
// algebra (trigonometricToExponentialMoments, src/mese/MESE_dynamic.h:38-40, and
// transform_dequantization_real, src/moment_prediction_coding.h:103-104), whose result every later step of
// prediction coding, the error-threshold count and the FP32 preparation depends on.
//
// The reference's CPU build takes cosf / sinf from the C library, and glibc's are not correctly rounded: over the
// floats of [-pi, pi] about one argument in a thousand comes out one ulp from the nearest float.  Two parts
// reproduce them exactly:
//
//  * the core (this file, one source for host and device): sin and cos of the float argument evaluated in double
//    and rounded once to float.  The argument is reduced by symmetry to |r| <= pi/4 (pi/2 and pi split into two
//    doubles, the first difference exact by Sterbenz's lemma), then Taylor polynomials of degree 19 (sin) and 20
//    (cos) by Horner's rule, whose truncation error is below 1e-19 on that interval.  Only double multiplications
//    and additions are used, each rounded on its own (the device form uses __dmul_rn / __dadd_rn, the host form is
//    compiled with -ffp-contract=off), so the host and device results are identical.
//  * an exception table (libm_trig_gen.cpp, run at build time on the machine whose C library the reference uses):
//    every float x of [-pi, pi] where the C library's sinf(x) or cosf(x) differs from the core's result.  Each
//    difference is one ulp (the generator checks this), so an entry is 16 bits: the low 12 bits of x plus, per
//    function, a "differs" flag and the direction of the ulp step.  Entries are bucketed by the other bits of x.
//
// Outside [-pi, pi] (never reached for the moments of a non-negative density, whose zeroth phase lies in
// [-pi/2, pi/2]) the device returns the double-precision functions rounded to float.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define MLT_HD __host__ __device__ __forceinline__
#else
#define MLT_HD inline
#endif

#if defined(__CUDA_ARCH__)
#define MLT_MUL(a, b) __dmul_rn((a), (b))
#define MLT_ADD(a, b) __dadd_rn((a), (b))
#else
#define MLT_MUL(a, b) ((a) * (b))
#define MLT_ADD(a, b) ((a) + (b))
#endif

namespace mraygb
{
namespace libm_trig
{

// Table layout (little endian):
//   Header, then uint32_t offsets[n_buckets + 1], then uint16_t entries[n_entries].
// Bucket of x: ((bits & 0x7fffffff) >> kShift) * 2 + (bits >> 31); inside a bucket, entries ascend by low bits.
constexpr uint32_t kMagic = 0x54544c4du; // "MLTT"
constexpr uint32_t kVersion = 1;
constexpr uint32_t kShift = 12;
constexpr uint32_t kLowMask = (1u << kShift) - 1u;
constexpr uint32_t kMaxAbsBits = 0x40490FDBu; // (float)pi, the largest magnitude covered
constexpr uint32_t kBuckets = ((kMaxAbsBits >> kShift) + 1u) * 2u;
constexpr uint16_t kSinDiffers = 1u << 12;
constexpr uint16_t kSinUp = 1u << 13; // C library bits = core bits + 1 (else - 1)
constexpr uint16_t kCosDiffers = 1u << 14;
constexpr uint16_t kCosUp = 1u << 15;

struct Header
{
    uint32_t magic, version, shift, n_buckets, n_entries, max_abs_bits, reserved0, reserved1;
};

MLT_HD uint32_t bucket_of(uint32_t bits) { return ((bits & 0x7fffffffu) >> kShift) * 2u + (bits >> 31); }
MLT_HD bool in_domain(uint32_t bits) { return (bits & 0x7fffffffu) <= kMaxAbsBits; }

// sin and cos of r in double, |r| <= pi/4
MLT_HD void taylor_sincos(double r, double &s, double &c)
{
    const double u = MLT_MUL(r, r);
    double ps = -0x1.2f49b46814157p-57; // -1/19!
    ps = MLT_ADD(MLT_MUL(ps, u), 0x1.952c77030ad4ap-49);  // 1/17!
    ps = MLT_ADD(MLT_MUL(ps, u), -0x1.ae7f3e733b81fp-41); // -1/15!
    ps = MLT_ADD(MLT_MUL(ps, u), 0x1.6124613a86d09p-33);  // 1/13!
    ps = MLT_ADD(MLT_MUL(ps, u), -0x1.ae64567f544e4p-26); // -1/11!
    ps = MLT_ADD(MLT_MUL(ps, u), 0x1.71de3a556c734p-19);  // 1/9!
    ps = MLT_ADD(MLT_MUL(ps, u), -0x1.a01a01a01a01ap-13); // -1/7!
    ps = MLT_ADD(MLT_MUL(ps, u), 0x1.1111111111111p-7);   // 1/5!
    ps = MLT_ADD(MLT_MUL(ps, u), -0x1.5555555555555p-3);  // -1/3!
    s = MLT_ADD(r, MLT_MUL(MLT_MUL(r, u), ps));
    double pc = 0x1.e542ba4020225p-62;                    // 1/20!
    pc = MLT_ADD(MLT_MUL(pc, u), -0x1.6827863b97d97p-53); // -1/18!
    pc = MLT_ADD(MLT_MUL(pc, u), 0x1.ae7f3e733b81fp-45);  // 1/16!
    pc = MLT_ADD(MLT_MUL(pc, u), -0x1.93974a8c07c9dp-37); // -1/14!
    pc = MLT_ADD(MLT_MUL(pc, u), 0x1.1eed8eff8d898p-29);  // 1/12!
    pc = MLT_ADD(MLT_MUL(pc, u), -0x1.27e4fb7789f5cp-22); // -1/10!
    pc = MLT_ADD(MLT_MUL(pc, u), 0x1.a01a01a01a01ap-16);  // 1/8!
    pc = MLT_ADD(MLT_MUL(pc, u), -0x1.6c16c16c16c17p-10); // -1/6!
    pc = MLT_ADD(MLT_MUL(pc, u), 0x1.5555555555555p-5);   // 1/4!
    c = MLT_ADD(MLT_ADD(1.0, MLT_MUL(-0.5, u)), MLT_MUL(MLT_MUL(u, u), pc));
}

// The core: sin and cos of x (|x| <= pi) in double, rounded once to float.
MLT_HD void core_sincosf(float xf, float &sf, float &cf)
{
    if (xf == 0.f) // sin(+-0) = +-0
    {
        sf = xf;
        cf = 1.f;
        return;
    }
    const double x = (double)xf;
    const double ax = x < 0.0 ? -x : x;
    double s, c;
    if (ax <= 0x1.921fb54442d18p-1) // pi/4
    {
        taylor_sincos(ax, s, c);
    }
    else if (ax <= 0x1.2d97c7f3321d2p+1) // 3 pi/4: sin(ax) = cos(pi/2 - ax), cos(ax) = sin(pi/2 - ax)
    {
        const double r = MLT_ADD(MLT_ADD(0x1.921fb54442d18p+0, -ax), 0x1.1a62633145c07p-54);
        double sr, cr;
        taylor_sincos(r, sr, cr);
        s = cr;
        c = sr;
    }
    else // sin(ax) = sin(pi - ax), cos(ax) = -cos(pi - ax)
    {
        const double r = MLT_ADD(MLT_ADD(0x1.921fb54442d18p+1, -ax), 0x1.1a62633145c07p-53);
        double sr, cr;
        taylor_sincos(r, sr, cr);
        s = sr;
        c = -cr;
    }
    if (x < 0.0)
        s = -s;
    sf = (float)s;
    cf = (float)c;
}

// Apply a table entry's corrections to the core's result (as bit patterns).
MLT_HD void apply_entry(uint16_t e, uint32_t &sbits, uint32_t &cbits)
{
    if (e & kSinDiffers)
        sbits = (e & kSinUp) ? sbits + 1u : sbits - 1u;
    if (e & kCosDiffers)
        cbits = (e & kCosUp) ? cbits + 1u : cbits - 1u;
}

// Find the entry of x (bits) in a table; returns 0 when x has none (entry 0 has no "differs" flag set).
MLT_HD uint16_t find_entry(const uint32_t *offsets, const uint16_t *entries, uint32_t bits)
{
    const uint32_t b = bucket_of(bits);
    const uint32_t lo = offsets[b], hi = offsets[b + 1];
    const uint32_t low = bits & kLowMask;
    for (uint32_t i = lo; i < hi; ++i)
    {
        const uint16_t e = entries[i];
        const uint32_t el = e & kLowMask;
        if (el == low)
            return e;
        if (el > low)
            break;
    }
    return 0;
}

} // namespace libm_trig
} // namespace mraygb
