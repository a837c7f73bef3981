// avbd_crmath.cuh — correctly rounded f32 sin, cos, asin and atan2, for host
// and device code.
//
// The reference computes these through the platform's f32 libm (Rust std
// f32::sin_cos / asin / atan2, crates/physics/src/avbd/rows.rs:115, :145,
// crates/physics/src/sequential_impulse/joints.rs:46).  Those libraries and
// CUDA's own differ from each other in the last bit on some arguments, and
// the AVBD step is ill-conditioned enough (penalties up to 1e10) that one
// ulp in a joint angle grows to 1e-4 in a pose within one step.  A correctly
// rounded result is unique, so every implementation that is correctly
// rounded — this one on the GPU, the oracle's on the host — returns the same
// float for every input.
//
// Method (Ziv, "Fast evaluation of elementary mathematical functions with
// correctly rounded last bit", ACM TOMS 17(3), 1991): evaluate in double with
// a relative error bound far below a float ulp; when the bound's interval
// rounds to one float, that float is the correctly rounded result; otherwise
// (about once in 2^24 arguments) evaluate again in double-double arithmetic
// (Dekker's two-sum / two-product) and round that.  Argument reduction of sin
// and cos by multiples of pi/2 is Payne and Hanek's ("Radian reduction for
// trigonometric functions", SIGNUM Newsletter 18(1), 1983): the float's
// 24-bit mantissa times a 192-bit window of the bits of 2/pi in integer
// arithmetic, exact for every float.  The series are the Taylor series of
// sin, cos, asin (for |x| <= 1/2; above, asin(x) = pi/2 - 2 asin(sqrt((1-x)/2)))
// and atan (after atan(t) = atan(c) + atan((t - c)/(1 + t c)), c = k/4).
// Every double operation is an explicitly rounded one (no contraction), so
// the double path gives the same bits in every build.  The constant tables
// were printed by gen_crmath_constants.py.
//
// Small arguments — the per-iteration rotations and joint twists of the step
// — first try a float stage: x + d with the Taylor correction d evaluated in
// float (|x| <= 1/16, or |y/x| <= 1/16 with x > 0 for atan2; t = y/x carried
// as t_hi + t_lo from the exact division remainder), the sum split exactly by
// Knuth's two-sum into s + e, and s accepted when |e| plus a bound of the
// evaluation error stays below half the gap from s to its neighbour on e's
// side (Ziv's test again, one level down).  The GB300's FP64 rate is a small
// fraction of its FP32 rate, and the float stage settles almost every call of
// the step; a rejected argument goes on to the double stage.
//
// The header also compiles as plain C++ (no CUDA compiler): the host
// definitions alone.
#pragma once
#ifdef __CUDACC__
#include <cuda_runtime.h>
#endif
#include <stdint.h>

#include <cmath>
#include <cstring>

namespace avbd {
namespace crm {

#ifdef __CUDA_ARCH__
#define CRM_MUL(a, b) __dmul_rn((a), (b))
#define CRM_ADD(a, b) __dadd_rn((a), (b))
#define CRM_SUB(a, b) __dsub_rn((a), (b))
#define CRM_DIV(a, b) __ddiv_rn((a), (b))
#define CRM_FMA(a, b, c) __fma_rn((a), (b), (c))
#define CRM_SQRT(a) __dsqrt_rn(a)
#define CRM_D2F(a) __double2float_rn(a)
#define CRM_T(name) name##_d
#else
#define CRM_MUL(a, b) ((a) * (b))
#define CRM_ADD(a, b) ((a) + (b))
#define CRM_SUB(a, b) ((a) - (b))
#define CRM_DIV(a, b) ((a) / (b))
#define CRM_FMA(a, b, c) std::fma((a), (b), (c))
#define CRM_SQRT(a) std::sqrt(a)
#define CRM_D2F(a) static_cast<float>(a)
#define CRM_T(name) name##_h
#endif
#ifdef __CUDACC__
#define CRM_HD __host__ __device__ __forceinline__
#define CRM_TABLE(type, name, ...)                      \
    static __constant__ const type name##_d[] = __VA_ARGS__; \
    static const type name##_h[] = __VA_ARGS__;
#else
#define CRM_HD static inline
#define CRM_TABLE(type, name, ...) static const type name##_h[] = __VA_ARGS__;
#endif

// bits 1..512 of 2/pi after the binary point
CRM_TABLE(uint64_t, k_two_over_pi, {
    0xa2f9836e4e441529ull,
    0xfc2757d1f534ddc0ull,
    0xdb6295993c439041ull,
    0xfe5163abdebbc561ull,
    0xb7246e3a424dd2e0ull,
    0x06492eea09d1921cull,
    0xfe1deb1cb129a73eull,
    0xe88235f52ebb4484ull
})
// pi/4, pi/2, pi, atan(1/4), atan(1/2), atan(3/4), atan(1) as double-doubles
CRM_TABLE(double, k_consts, {
    0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55,
    0x1.921fb54442d18p+0, 0x1.1a62633145c07p-54,
    0x1.921fb54442d18p+1, 0x1.1a62633145c07p-53,
    0x1.f5b75f92c80ddp-3, 0x1.8ab6e3cf7afbdp-57,
    0x1.dac670561bb4fp-2, 0x1.a2b7f222f65e2p-56,
    0x1.4978fa3269ee1p-1, 0x1.2419a87f2a458p-56,
    0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55
})
// Taylor coefficients (hi, lo): sin (-1)^n/(2n+1)!, cos (-1)^n/(2n)!, n >= 1
CRM_TABLE(double, k_sin, {
    -0x1.5555555555555p-3, -0x1.5555555555555p-57,
    0x1.1111111111111p-7, 0x1.1111111111111p-63,
    -0x1.a01a01a01a01ap-13, -0x1.a01a01a01a01ap-73,
    0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73,
    -0x1.ae64567f544e4p-26, 0x1.c062e06d1f209p-80,
    0x1.6124613a86d09p-33, 0x1.f28e0cc748ebep-87,
    -0x1.ae7f3e733b81fp-41, -0x1.1d8656b0ee8cbp-97,
    0x1.952c77030ad4ap-49, 0x1.ac981465ddc6cp-103,
    -0x1.2f49b46814157p-57, -0x1.2650f61dbdcb4p-112,
    0x1.71b8ef6dcf572p-66, -0x1.d043ae40c4647p-120,
    -0x1.761b41316381ap-75, 0x1.3423c7d91404fp-130,
    0x1.3f3ccdd165fa9p-84, -0x1.58ddadf344487p-139,
    -0x1.d1ab1c2dccea3p-94, -0x1.054d0c78aea14p-149,
    0x1.259f98b4358adp-103, 0x1.eaf8c39dd9bc5p-157,
    -0x1.434d2e783f5bcp-113, -0x1.0b87b91be9affp-167
})
CRM_TABLE(double, k_cos, {
    -0x1.0000000000000p-1, 0x0.0p+0,
    0x1.5555555555555p-5, 0x1.5555555555555p-59,
    -0x1.6c16c16c16c17p-10, 0x1.f49f49f49f49fp-65,
    0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76,
    -0x1.27e4fb7789f5cp-22, -0x1.cbbc05b4fa99ap-76,
    0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83,
    -0x1.93974a8c07c9dp-37, -0x1.05d6f8a2efd1fp-92,
    0x1.ae7f3e733b81fp-45, 0x1.1d8656b0ee8cbp-101,
    -0x1.6827863b97d97p-53, -0x1.eec01221a8b0bp-107,
    0x1.e542ba4020225p-62, 0x1.ea72b4afe3c2fp-120,
    -0x1.0ce396db7f853p-70, 0x1.aebcdbd20331cp-124,
    0x1.f2cf01972f578p-80, -0x1.9ada5fcc1ab14p-135,
    -0x1.88e85fc6a4e5ap-89, 0x1.71c37ebd16540p-143,
    0x1.0a18a2635085dp-98, 0x1.b9e2e28e1aa54p-153,
    -0x1.3932c5047d60ep-108, -0x1.832b7b530a627p-162
})
// asin (2n)!/(4^n (n!)^2 (2n+1)), atan (-1)^n/(2n+1), n >= 1
CRM_TABLE(double, k_asin, {
    0x1.5555555555555p-3, 0x1.5555555555555p-57,
    0x1.3333333333333p-4, 0x1.999999999999ap-59,
    0x1.6db6db6db6db7p-5, -0x1.2492492492492p-60,
    0x1.f1c71c71c71c7p-6, 0x1.c71c71c71c71cp-62,
    0x1.6e8ba2e8ba2e9p-6, -0x1.1745d1745d174p-60,
    0x1.1c4ec4ec4ec4fp-6, -0x1.d89d89d89d89ep-61,
    0x1.c99999999999ap-7, -0x1.999999999999ap-61,
    0x1.7a87878787878p-7, 0x1.e1e1e1e1e1e1ep-61,
    0x1.3fde50d79435ep-7, 0x1.435e50d79435ep-61,
    0x1.12ef3cf3cf3cfp-7, 0x1.e79e79e79e79ep-62,
    0x1.df3bd37a6f4dfp-8, -0x1.90b21642c8591p-62,
    0x1.a6863d70a3d71p-8, -0x1.70a3d70a3d70ap-62,
    0x1.782dda12f684cp-8, -0x1.2f684bda12f68p-63,
    0x1.51ba308d3dcb1p-8, -0x1.cb08d3dcb08d4p-62,
    0x1.31683bdef7bdfp-8, -0x1.0842108421084p-65,
    0x1.15ee9d45d1746p-8, -0x1.745d1745d1746p-63,
    0x1.fcaf8fb6db6dbp-9, 0x1.b6db6db6db6dbp-63,
    0x1.d3d2a8e0dd67dp-9, -0x1.d67c8a60dd67dp-63,
    0x1.b026f57b13b14p-9, -0x1.3b13b13b13b14p-63,
    0x1.90cb77f60c7cep-9, 0x1.8f9c18f9c18fap-66,
    0x1.750de64d7d05fp-9, 0x1.05f417d05f418p-63,
    0x1.5c5f56efaaaabp-9, -0x1.5555555555555p-63,
    0x1.464c0950f7d47p-9, -0x1.882b931057262p-64,
    0x1.3275586c5f2f0p-9, 0x1.4e5e0a72f0539p-63,
    0x1.208d3570ae5a6p-9, -0x1.6969696969697p-63,
    0x1.1052bc5fa960ap-9, -0x1.5bc609a90e7d9p-63,
    0x1.018f963c229bfp-9, -0x1.4f2094f2094f2p-64,
    0x1.e82be60d9127ep-10, -0x1.f7047dc11f704p-65,
    0x1.cf7dea5b6e830p-10, -0x1.15b1e5f75270dp-64,
    0x1.b8d2e5667ce6cp-10, 0x1.0c9714fbcda3bp-66,
    0x1.a3f1ef82137eep-10, 0x1.c71c71c71c71cp-65,
    0x1.90a9f747db95dp-10, -0x1.6a56a56a56a57p-65,
    0x1.7ed079ed4c037p-10, -0x1.03d226357e16fp-66,
    0x1.6e40790442038p-10, 0x1.a6f4de9bd37a7p-67,
    0x1.5ed9a0bd901b6p-10, -0x1.040e6c2b4481dp-64,
    0x1.507f94c2470bdp-10, 0x1.56070381c0e07p-65,
    0x1.43195bf54e5d7p-10, -0x1.b9e4b17e4b17ep-64,
    0x1.3690e51f04536p-10, 0x1.9d9745d1745d1p-64,
    0x1.2ad29fcd49d54p-10, 0x1.82fbf309b8b57p-64,
    0x1.1fcd25ae4a26ep-10, 0x1.ca730fcd6e9e0p-65,
    0x1.1570f16ece10ap-10, 0x1.a9e4bf3a9a378p-64,
    0x1.0bb020bc1eaa0p-10, 0x1.8c4b078787878p-64,
    0x1.027e3f7fcd8bfp-10, 0x1.67f632c234f73p-64,
    0x1.f3a03591c2915p-11, 0x1.22b2be05c0b81p-65,
    0x1.e337343f5c1f5p-11, 0x1.ef13d589d89d9p-65,
    0x1.d3af3c78ce2e4p-11, 0x1.8eec64a5294a5p-68,
    0x1.c4f7c88f08b5ep-11, 0x1.4d45526bca1afp-66,
    0x1.b701d9e1f038ep-11, -0x1.2bb23e09fab8cp-65,
    0x1.a9bfcd93a26fdp-11, 0x1.437ecd445d174p-67,
    0x1.9d2536c99619ap-11, -0x1.fd25b093f5dc8p-70,
    0x1.9126bdad380c3p-11, -0x1.b9945c5ec813ep-65,
    0x1.85ba027ef48d7p-11, -0x1.dd7be76e2e2bep-65,
    0x1.7ad5842a041b9p-11, 0x1.2880cf6e197edp-65,
    0x1.707089ddf7dc4p-11, 0x1.f99269e145605p-65,
    0x1.66830f45c9d3fp-11, -0x1.ad72816baa298p-68,
    0x1.5d05b303d708cp-11, 0x1.8340a07dbd9c1p-66
})
CRM_TABLE(double, k_atan, {
    -0x1.5555555555555p-2, -0x1.5555555555555p-56,
    0x1.999999999999ap-3, -0x1.999999999999ap-57,
    -0x1.2492492492492p-3, -0x1.2492492492492p-57,
    0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58,
    -0x1.745d1745d1746p-4, 0x1.745d1745d1746p-59,
    0x1.3b13b13b13b14p-4, -0x1.3b13b13b13b14p-58,
    -0x1.1111111111111p-4, -0x1.1111111111111p-60,
    0x1.e1e1e1e1e1e1ep-5, 0x1.e1e1e1e1e1e1ep-61,
    -0x1.af286bca1af28p-5, -0x1.af286bca1af28p-59,
    0x1.8618618618618p-5, 0x1.8618618618618p-59,
    -0x1.642c8590b2164p-5, -0x1.642c8590b2164p-60,
    0x1.47ae147ae147bp-5, -0x1.eb851eb851eb8p-61,
    -0x1.2f684bda12f68p-5, -0x1.2f684bda12f68p-59,
    0x1.1a7b9611a7b96p-5, 0x1.1a7b9611a7b96p-61,
    -0x1.0842108421084p-5, -0x1.0842108421084p-60,
    0x1.f07c1f07c1f08p-6, -0x1.f07c1f07c1f08p-61,
    -0x1.d41d41d41d41dp-6, -0x1.0750750750750p-60,
    0x1.bacf914c1bad0p-6, -0x1.bacf914c1bad0p-60,
    -0x1.a41a41a41a41ap-6, -0x1.0690690690690p-60,
    0x1.8f9c18f9c18fap-6, -0x1.f3831f3831f38p-61,
    -0x1.7d05f417d05f4p-6, -0x1.7d05f417d05f4p-62,
    0x1.6c16c16c16c17p-6, -0x1.f49f49f49f49fp-61,
    -0x1.5c9882b931057p-6, -0x1.310572620ae4cp-61,
    0x1.4e5e0a72f0539p-6, 0x1.e0a72f0539783p-60
})

struct DD {
    double hi, lo;
};
CRM_HD DD two_sum(double a, double b) {
    double s = CRM_ADD(a, b);
    double bb = CRM_SUB(s, a);
    double e = CRM_ADD(CRM_SUB(a, CRM_SUB(s, bb)), CRM_SUB(b, bb));
    return {s, e};
}
CRM_HD DD fast_two_sum(double a, double b) {  // |a| >= |b| or a == 0
    double s = CRM_ADD(a, b);
    return {s, CRM_SUB(b, CRM_SUB(s, a))};
}
CRM_HD DD dd_add(DD x, DD y) {
    DD s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, CRM_ADD(s.lo, CRM_ADD(x.lo, y.lo)));
}
CRM_HD DD dd_neg(DD x) { return {-x.hi, -x.lo}; }
CRM_HD DD dd_mul(DD x, DD y) {
    double p = CRM_MUL(x.hi, y.hi);
    double e = CRM_FMA(x.hi, y.hi, -p);
    e = CRM_ADD(e, CRM_FMA(x.hi, y.lo, CRM_MUL(x.lo, y.hi)));
    return fast_two_sum(p, e);
}
CRM_HD DD dd_div(DD x, DD y) {
    double q1 = CRM_DIV(x.hi, y.hi);
    DD r = dd_add(x, dd_neg(dd_mul(y, DD{q1, 0.0})));
    double q2 = CRM_DIV(r.hi, y.hi);
    return fast_two_sum(q1, q2);
}
CRM_HD DD cst(int i) { return {CRM_T(k_consts)[2 * i], CRM_T(k_consts)[2 * i + 1]}; }
enum { C_PI4 = 0, C_PI2 = 1, C_PI = 2, C_ATAN_Q = 3 };  // atan(k/4) at C_ATAN_Q + k - 1

CRM_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
CRM_HD bool sign_bit(float f) { return (f2u(f) >> 31) != 0u; }
CRM_HD float next_up(float f) { return nextafterf(f, INFINITY); }
CRM_HD float next_down(float f) { return nextafterf(f, -INFINITY); }

// Round hi + lo (|lo| <= ulp(hi)) to the nearest float.
CRM_HD float dd_to_float(DD v) {
    float f = CRM_D2F(v.hi);
    double fd = (double)f;
    double d = CRM_ADD(CRM_SUB(v.hi, fd), v.lo);
    if (d > 0.0) {
        float u = next_up(f);
        double mid = CRM_MUL(CRM_SUB((double)u, fd), 0.5);
        if (d > mid) return u;
    } else if (d < 0.0) {
        float u = next_down(f);
        double mid = CRM_MUL(CRM_SUB(fd, (double)u), 0.5);
        if (-d > mid) return u;
    }
    return f;
}
// Ziv's rounding test: y approximates the result with |error| <= err.
CRM_HD bool rounds_to(double y, double err, float& out) {
    float a = CRM_D2F(CRM_SUB(y, err)), b = CRM_D2F(CRM_ADD(y, err));
    out = a;
#ifdef AVBD_CRMATH_TEST_SLOW  // tests: take the double-double path everywhere
    return false;
#else
    return a == b;
#endif
}
CRM_HD double err_bound(double y, double rel) { return CRM_ADD(CRM_MUL(fabs(y), rel), 0x1p-1070); }

// Terms of each series for |z| below a class bound (z = x^2); the tail is
// below 2^-60 (double path) or 2^-112 (double-double path) of the leading
// term.  Classes: z <= 2^-20, 2^-12, 2^-8, 2^-5, 2^-3, 2^-2, (pi/4)^2.
CRM_HD int z_class(double z) {
    return z <= 0x1p-20 ? 0 : z <= 0x1p-12 ? 1 : z <= 0x1p-8 ? 2 : z <= 0x1p-5 ? 3 : z <= 0x1p-3 ? 4 : z <= 0x1p-2 ? 5 : 6;
}
// series: 0 sin, 1 cos, 2 asin, 3 atan; 7 classes each
CRM_TABLE(int8_t, k_terms_fast, {2, 3, 4, 5, 6, 7, 8, 2, 3, 4, 6, 7, 7, 9, 2, 4, 6, 10, 17, 25, 25, 2, 4, 7, 11, 11, 11, 11})
CRM_TABLE(int8_t, k_terms_slow,
          {4, 6, 7, 9, 11, 12, 13, 4, 6, 8, 10, 11, 12, 14, 5, 8, 13, 20, 34, 51, 51, 5, 8, 13, 21, 21, 21, 21})
CRM_HD int terms(int series, int cls, bool slow) {
    return slow ? CRM_T(k_terms_slow)[series * 7 + cls] : CRM_T(k_terms_fast)[series * 7 + cls];
}
// Horner over coefficient table c (hi, lo pairs), terms n = 1..N: sum c_n z^(n-1)
CRM_HD double horner(const double* c, int n, double z) {
    double p = c[2 * (n - 1)];
    for (int k = n - 2; k >= 0; k--) p = CRM_FMA(p, z, c[2 * k]);
    return p;
}
CRM_HD DD horner_dd(const double* c, int n, DD z) {
    DD p{c[2 * (n - 1)], c[2 * (n - 1) + 1]};
    for (int k = n - 2; k >= 0; k--) p = dd_add(dd_mul(p, z), DD{c[2 * k], c[2 * k + 1]});
    return p;
}

// ---- float stage ----------------------------------------------------------------
#ifdef __CUDA_ARCH__
#define CRF_MUL(a, b) __fmul_rn((a), (b))
#define CRF_ADD(a, b) __fadd_rn((a), (b))
#define CRF_SUB(a, b) __fsub_rn((a), (b))
#define CRF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define CRF_DIV(a, b) __fdiv_rn((a), (b))
#else
#define CRF_MUL(a, b) ((a) * (b))
#define CRF_ADD(a, b) ((a) + (b))
#define CRF_SUB(a, b) ((a) - (b))
#define CRF_FMA(a, b, c) std::fma((a), (b), (c))
#define CRF_DIV(a, b) ((a) / (b))
#endif
// s + e = a + b exactly (Knuth's two-sum; round to nearest, no overflow)
CRM_HD void two_sum_f(float a, float b, float& s, float& e) {
    s = CRF_ADD(a, b);
    float bb = CRF_SUB(s, a);
    e = CRF_ADD(CRF_SUB(a, CRF_SUB(s, bb)), CRF_SUB(b, bb));
}
// The value lies in [s + e - err, s + e + err], s = fl(s + e): s is its
// correctly rounded float when neither end crosses the midpoint between s
// and its neighbour on that side (the gaps below and above s differ at a
// power of two).  The comparisons keep a 1% margin over the rounding of
// e +- err.
CRM_HD bool float_stage_ok(float s, float e, float err) {
#ifdef AVBD_CRMATH_TEST_DOUBLE  // tests: skip the float stage
    return false;
#else
    if (!(fabsf(s) < 3.0e38f) || fabsf(s) < 0x1p-100f) return false;
    const float up = CRF_MUL(CRF_SUB(next_up(s), s), 0.5f);    // exact
    const float dn = CRF_MUL(CRF_SUB(s, next_down(s)), 0.5f);  // exact
    return CRF_MUL(CRF_ADD(e, err), 1.01f) < up && CRF_MUL(CRF_SUB(err, e), 1.01f) < dn;
#endif
}
// x + x^3 (c1 + z (c2 + z c3)), z = x^2, |x| <= 1/16: the sin and asin
// stages.  The series' next term is below 2^-36 |x|.
CRM_HD bool odd_stage(float x, float c1, float c2, float c3, float& out) {
    const float z = CRF_MUL(x, x);
    const float p = CRF_FMA(CRF_FMA(c3, z, c2), z, c1);
    const float d = CRF_MUL(CRF_MUL(x, z), p);
    float s, e;
    two_sum_f(x, d, s, e);
    const float err = CRF_FMA(fabsf(d), 0x1p-20f, CRF_MUL(fabsf(x), 0x1p-36f));
    out = s;
    return float_stage_ok(s, e, err);
}
CRM_HD bool sin_stage(float x, float& out) {
    return fabsf(x) <= 0.0625f && odd_stage(x, -0x1.555556p-3f, 0x1.111112p-7f, -0x1.a01a02p-13f, out);
}
// 1 + z (-1/2 + z (1/24 - z/720)), |x| <= 1/16; next term below 2^-47
CRM_HD bool cos_stage(float x, float& out) {
    if (!(fabsf(x) <= 0.0625f)) return false;
    const float z = CRF_MUL(x, x);
    const float d = CRF_MUL(z, CRF_FMA(CRF_FMA(-0x1.6c16c2p-10f, z, 0x1.555556p-5f), z, -0.5f));
    float s, e;
    two_sum_f(1.0f, d, s, e);
    const float err = CRF_FMA(fabsf(d), 0x1p-20f, 0x1p-45f);
    out = s;
    return float_stage_ok(s, e, err);
}
CRM_HD bool asin_stage(float x, float& out) {
    // asin: x + x^3 (1/6 + z (3/40 + z 15/336)); the next term is below 2^-37 |x|
    return fabsf(x) <= 0.0625f && odd_stage(x, 0x1.555556p-3f, 0x1.333334p-4f, 0x1.6db6dcp-5f, out);
}
// atan2(y, x) for x > 0, |y| <= x/16: t = y/x = th + tl, atan(t) = t + t^3 (-1/3
// + z (1/5 - z/7)); the next term is below 2^-35 |t|.
CRM_HD bool atan2_stage(float y, float x, float& out) {
    // y/x's remainder y - th x is exact only if it stays above the subnormal range
    if (!(x > 0.0f) || !(x < 3.0e38f) || !(fabsf(y) <= CRF_MUL(x, 0.0625f)) || fabsf(y) < 0x1p-90f) return false;
    const float th = CRF_DIV(y, x);
    const float tl = CRF_DIV(CRF_FMA(-th, x, y), x);  // the remainder y - th x is exact
    const float z = CRF_MUL(th, th);
    const float p = CRF_FMA(CRF_FMA(-0x1.24924ap-3f, z, 0x1.99999ap-3f), z, -0x1.555556p-2f);
    const float tail = CRF_MUL(CRF_MUL(th, z), p);
    const float d = CRF_ADD(tl, tail);
    float s, e;
    two_sum_f(th, d, s, e);
    // the tail's rounding, the sum's, and the tail taken at th instead of t
    // (|t - th| <= 2^-24 |th|, the tail's slope |t|^2 <= 2^-8) with the series' rest
    const float err = CRF_FMA(CRF_ADD(fabsf(tail), fabsf(tl)), 0x1p-20f, CRF_MUL(fabsf(th), 0x1p-31f));
    out = s;
    return float_stage_ok(s, e, err);
}

// ---- sin, cos -----------------------------------------------------------------
CRM_HD uint64_t mul_hi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
// bits [pos, pos + 64) of the 256-bit integer w (w[0] least significant)
CRM_HD uint64_t bits64(const uint64_t w[5], int pos) {
    int i = pos >> 6, s = pos & 63;
    uint64_t lo = w[i];
    uint64_t hi = i + 1 < 5 ? w[i + 1] : 0u;
    return s ? (lo >> s) | (hi << (64 - s)) : lo;
}
// |x| = r + j pi/2 with |r| <= pi/4 (plus a rounding margin), for finite
// |x| >= pi/4: Payne-Hanek on the exact float.  Returns j mod 4.
CRM_HD int reduce_pio2(float ax, DD& r) {
    const uint32_t u = f2u(ax);
    const int ex = (int)((u >> 23) & 255u);
    const uint64_t m = (uint64_t)((u & 0x7fffffu) | 0x800000u);
    const int e = ex - 150;  // ax = m 2^e
    const int s = e - 2 > 0 ? e - 2 : 0;  // bits of 2/pi up to s give multiples of 4
    const int wi = s >> 6, sh = s & 63;
    const uint64_t* T = CRM_T(k_two_over_pi);
    uint64_t t0 = T[wi], t1 = T[wi + 1], t2 = T[wi + 2], t3 = T[wi + 3];
    uint64_t W0 = sh ? (t0 << sh) | (t1 >> (64 - sh)) : t0;  // bits s+1 .. s+64
    uint64_t W1 = sh ? (t1 << sh) | (t2 >> (64 - sh)) : t1;
    uint64_t W2 = sh ? (t2 << sh) | (t3 >> (64 - sh)) : t2;
    // P = m * (W0 W1 W2), 256 bits, little-endian words
    uint64_t p[5];
    uint64_t l2 = m * W2, h2 = mul_hi64(m, W2);
    uint64_t l1 = m * W1, h1 = mul_hi64(m, W1);
    uint64_t l0 = m * W0, h0 = mul_hi64(m, W0);
    p[0] = l2;
    p[1] = l1 + h2;
    uint64_t c1 = p[1] < l1 ? 1u : 0u;
    p[2] = l0 + h1;
    uint64_t c2 = p[2] < l0 ? 1u : 0u;
    p[2] += c1;
    c2 += (p[2] < c1) ? 1u : 0u;
    p[3] = h0 + c2;
    p[4] = 0;
    // ax (2/pi) = P 2^(e - s - 192): the binary point sits at bit q of P
    const int q = 192 - (e - s);
    int j = (int)(bits64(p, q) & 3u);
    uint64_t fh = bits64(p, q - 64), fl = bits64(p, q - 128);  // 128 fraction bits
    double sign = 1.0;
    if (fh >> 63) {  // fraction >= 1/2: take r from the next multiple
        j = (j + 1) & 3;
        fl = ~fl + 1u;
        fh = ~fh + (fl == 0u ? 1u : 0u);
        sign = -1.0;
    }
    // the 128-bit fraction as an exact sum of three doubles, then a double-double
    double d1 = CRM_MUL((double)(fh >> 11), 0x1p-53);
    double d2 = CRM_MUL((double)(((fh & 0x7ffu) << 42) | (fl >> 22)), 0x1p-106);
    double d3 = CRM_MUL((double)(fl & 0x3fffffu), 0x1p-128);
    DD f = dd_add(two_sum(d1, d2), DD{d3, 0.0});
    r = dd_mul(f, cst(C_PI2));
    r.hi *= sign;
    r.lo *= sign;
    return j;
}
// The double-double evaluations run about once in 2^24 arguments: kept out
// of line so that the fast paths stay small.
#ifdef __CUDACC__
#define CRM_SLOW static __host__ __device__ __noinline__
#else
#define CRM_SLOW static __attribute__((noinline))
#endif
CRM_SLOW float sincos_slow(DD r, bool use_sin, double sgn) {
    DD zz = dd_mul(r, r);
    int n = terms(use_sin ? 0 : 1, z_class(zz.hi), true);
    DD v;
    if (use_sin) {
        DD p = horner_dd(CRM_T(k_sin), n, zz);
        v = dd_add(r, dd_mul(dd_mul(r, zz), p));
    } else {
        DD p = horner_dd(CRM_T(k_cos), n, zz);
        v = dd_add(DD{1.0, 0.0}, dd_mul(zz, p));
    }
    v.hi *= sgn;
    v.lo *= sgn;
    return dd_to_float(v);
}
// sin (want_sin) or cos of |x| reduced to r, quadrant j
CRM_HD float sincos_finish(DD r, int j, bool want_sin, float xsign) {
    // sin(x) = [s, c, -s, -c][j], cos(x) = [c, -s, -c, s][j]
    const int k = want_sin ? j : (j + 1) & 3;
    const bool use_sin = (k & 1) == 0;
    const bool neg = k >= 2;
    const double rh = r.hi, rl = r.lo;
    const double z = CRM_MUL(rh, rh);
    const int cls = z_class(z);
    double y;
    if (use_sin) {
        double p = horner(CRM_T(k_sin), terms(0, cls, false), z);
        y = CRM_FMA(CRM_MUL(rh, z), p, rh);
        y = CRM_ADD(y, rl);  // sin(rh + rl) = sin(rh) + rl (1 - rh^2/2 ...)
    } else {
        double p = horner(CRM_T(k_cos), terms(1, cls, false), z);
        y = CRM_FMA(z, p, 1.0);
        y = CRM_FMA(-rl, rh, y);  // cos(rh + rl) = cos(rh) - rl sin(rh) ...
    }
    double sgn = (neg ? -1.0 : 1.0) * (want_sin ? (double)xsign : 1.0);
    y = CRM_MUL(y, sgn);
    float out;
    if (rounds_to(y, err_bound(y, 0x1p-49), out)) return out;
    return sincos_slow(r, use_sin, sgn);
}
CRM_HD void reduce(float x, DD& r, int& j) {
    float ax = fabsf(x);
    if (ax < 0.785398f) {  // below pi/4: no reduction
        r = DD{(double)ax, 0.0};
        j = 0;
    } else {
        j = reduce_pio2(ax, r);
    }
}
CRM_HD float sinf(float x) {
    if (!(fabsf(x) <= 3.4028235e38f)) return x - x;  // NaN for NaN and infinities
    if (x == 0.0f) return x;
    float f;
    if (sin_stage(x, f)) return f;
    DD r;
    int j;
    reduce(x, r, j);
    return sincos_finish(r, j, true, x < 0.0f ? -1.0f : 1.0f);
}
CRM_HD float cosf(float x) {
    if (!(fabsf(x) <= 3.4028235e38f)) return x - x;
    if (x == 0.0f) return 1.0f;
    float f;
    if (cos_stage(x, f)) return f;
    DD r;
    int j;
    reduce(x, r, j);
    return sincos_finish(r, j, false, 1.0f);
}
CRM_HD void sincosf(float x, float* s, float* c) {
    if (!(fabsf(x) <= 3.4028235e38f)) {
        *s = *c = x - x;
        return;
    }
    if (x == 0.0f) {
        *s = x;
        *c = 1.0f;
        return;
    }
    float fs, fc;
    const bool ks = sin_stage(x, fs), kc = cos_stage(x, fc);
    if (ks && kc) {
        *s = fs;
        *c = fc;
        return;
    }
    DD r;
    int j;
    reduce(x, r, j);
    *s = ks ? fs : sincos_finish(r, j, true, x < 0.0f ? -1.0f : 1.0f);
    *c = kc ? fc : sincos_finish(r, j, false, 1.0f);
}

// ---- asin ------------------------------------------------------------------------
CRM_SLOW float asin_slow(float ax, double sgn);
CRM_HD float asinf(float x) {
    const float ax = fabsf(x);
    if (!(ax <= 1.0f)) return (x - x) / (x - x);  // NaN for NaN and |x| > 1
    if (x == 0.0f) return x;
    float f;
    if (asin_stage(x, f)) return f;
    const double sgn = x < 0.0f ? -1.0 : 1.0;
    const double a = (double)ax;
    double y;
    if (ax <= 0.5f) {
        double z = CRM_MUL(a, a);  // exact: 48-bit product
        double p = horner(CRM_T(k_asin), terms(2, z_class(z), false), z);
        y = CRM_FMA(CRM_MUL(a, z), p, a);
    } else {
        double z = CRM_MUL(CRM_SUB(1.0, a), 0.5);  // exact
        double s = CRM_SQRT(z);
        double p = horner(CRM_T(k_asin), terms(2, z_class(z), false), z);
        double as = CRM_FMA(CRM_MUL(s, z), p, s);
        DD h = cst(C_PI2);
        y = CRM_ADD(CRM_FMA(-2.0, as, h.hi), h.lo);
    }
    y = CRM_MUL(y, sgn);
    float out;
    if (rounds_to(y, err_bound(y, 0x1p-48), out)) return out;
    return asin_slow(ax, sgn);
}
CRM_SLOW float asin_slow(float ax, double sgn) {
    const double a = (double)ax;
    DD v;
    if (ax <= 0.5f) {
        DD xa{a, 0.0};
        DD z = dd_mul(xa, xa);
        DD p = horner_dd(CRM_T(k_asin), terms(2, z_class(z.hi), true), z);
        v = dd_add(xa, dd_mul(dd_mul(xa, z), p));
    } else {
        double z = CRM_MUL(CRM_SUB(1.0, a), 0.5);
        double sh = CRM_SQRT(z);
        double sl = sh > 0.0 ? CRM_DIV(CRM_FMA(-sh, sh, z), CRM_MUL(2.0, sh)) : 0.0;
        DD s = fast_two_sum(sh, sl), zz{z, 0.0};
        DD p = horner_dd(CRM_T(k_asin), terms(2, z_class(z), true), zz);
        DD as = dd_add(s, dd_mul(dd_mul(s, zz), p));
        v = dd_add(cst(C_PI2), dd_mul(DD{-2.0, 0.0}, as));
    }
    v.hi *= sgn;
    v.lo *= sgn;
    return dd_to_float(v);
}

// ---- atan2 -----------------------------------------------------------------------
CRM_SLOW float atan2_slow(double num, double den, int k, bool swap, bool xneg, float sy);
CRM_HD float atan2f(float y, float x) {
    if (x != x || y != y) return x + y;
    const float ax = fabsf(x), ay = fabsf(y);
    const float sy = sign_bit(y) ? -1.0f : 1.0f;
    const bool xneg = sign_bit(x);
    const float INF = INFINITY;
    if (ay == 0.0f) return xneg ? sy * dd_to_float(cst(C_PI)) : sy * 0.0f;
    if (ax == 0.0f) return sy * dd_to_float(cst(C_PI2));
    if (ay == INF || ax == INF) {
        if (ay == INF && ax == INF) {
            DD v = xneg ? dd_add(cst(C_PI), dd_neg(cst(C_PI4))) : cst(C_PI4);
            return sy * dd_to_float(v);
        }
        if (ay == INF) return sy * dd_to_float(cst(C_PI2));
        return xneg ? sy * dd_to_float(cst(C_PI)) : sy * 0.0f;
    }
    float f;
    if (atan2_stage(y, x, f)) return f;
    const bool swap = ay > ax;
    const double num = swap ? (double)ax : (double)ay, den = swap ? (double)ay : (double)ax;
    const double t = CRM_DIV(num, den);  // [0, 1]
    const int k = (int)rint(CRM_MUL(t, 4.0));
    const double c = CRM_MUL((double)k, 0.25);
    double u = k ? CRM_DIV(CRM_SUB(t, c), CRM_FMA(t, c, 1.0)) : t;
    double z = CRM_MUL(u, u);
    double p = horner(CRM_T(k_atan), terms(3, z_class(z), false), z);
    double at = CRM_FMA(CRM_MUL(u, z), p, u);
    if (k) {
        DD b = cst(C_ATAN_Q + k - 1);
        at = CRM_ADD(b.hi, CRM_ADD(at, b.lo));
    }
    double res = at;
    if (swap) {
        DD h = cst(C_PI2);
        res = CRM_ADD(CRM_SUB(h.hi, res), h.lo);
    }
    if (xneg) {
        DD h = cst(C_PI);
        res = CRM_ADD(CRM_SUB(h.hi, res), h.lo);
    }
    res = CRM_MUL(res, (double)sy);
    float out;
    if (rounds_to(res, err_bound(res, 0x1p-47), out)) return out;
    return atan2_slow(num, den, k, swap, xneg, sy);
}
CRM_SLOW float atan2_slow(double num, double den, int k, bool swap, bool xneg, float sy) {
    const double c = CRM_MUL((double)k, 0.25);
    DD td = dd_div(DD{num, 0.0}, DD{den, 0.0});
    DD ud = k ? dd_div(dd_add(td, DD{-c, 0.0}), dd_add(DD{1.0, 0.0}, dd_mul(td, DD{c, 0.0}))) : td;
    DD zd = dd_mul(ud, ud);
    DD pd = horner_dd(CRM_T(k_atan), terms(3, z_class(zd.hi), true), zd);
    DD v = dd_add(ud, dd_mul(dd_mul(ud, zd), pd));
    if (k) v = dd_add(cst(C_ATAN_Q + k - 1), v);
    if (swap) v = dd_add(cst(C_PI2), dd_neg(v));
    if (xneg) v = dd_add(cst(C_PI), dd_neg(v));
    v.hi *= (double)sy;
    v.lo *= (double)sy;
    return dd_to_float(v);
}

}  // namespace crm
}  // namespace avbd
