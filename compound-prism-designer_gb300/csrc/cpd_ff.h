// cpd_ff.h -- float-float ("double-single") arithmetic for the entropy sums.
//
// On this GPU an f64 log2 costs about 290 FP32 log2s, so the p log2 p terms of the
// entropy are formed in float-float arithmetic on the FP32 pipe: a value is an
// unevaluated sum hi + lo of two floats (~48-bit significand). The error-free
// transformations are Knuth's two-sum and the fused-multiply-add two-product; log2 is
// Tang's table-driven method: log2(c) = e + log2(c_i) + log2(1 + r) with c_i = 1 + i/256
// the nearest table point below the mantissa and r = (m - c_i)/c_i < 2^-8, the series
// log2(1 + r) = (r - r^2/2 + r^3/3 - ...)/ln 2 taking its leading term in float-float
// and the rest in FP32. Absolute error of log2 is below 1e-12 (tested against the host
// f64 log2).
#pragma once

#include <cstdint>
#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define CPD_FF_HD __host__ __device__ __forceinline__
#else
#define CPD_FF_HD inline
#endif

namespace cpd {
namespace ff {

struct F2 {
    float hi, lo;
};

CPD_FF_HD float fmaf_(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
CPD_FF_HD float add_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);  // not contracted or reassociated
#else
    volatile float s = a + b;
    return s;
#endif
}
CPD_FF_HD float sub_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    volatile float s = a - b;
    return s;
#endif
}
CPD_FF_HD float mul_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    volatile float s = a * b;
    return s;
#endif
}

// Knuth two-sum: s + e == a + b exactly.
CPD_FF_HD F2 two_sum(float a, float b)
{
    const float s = add_rn(a, b);
    const float bb = sub_rn(s, a);
    const float e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
    return F2{s, e};
}
// |a| >= |b|
CPD_FF_HD F2 fast_two_sum(float a, float b)
{
    const float s = add_rn(a, b);
    return F2{s, sub_rn(b, sub_rn(s, a))};
}
CPD_FF_HD F2 add(F2 a, F2 b)
{
    F2 s = two_sum(a.hi, b.hi);
    const float lo = add_rn(s.lo, add_rn(a.lo, b.lo));
    return fast_two_sum(s.hi, lo);
}
CPD_FF_HD F2 add_f(F2 a, float b)
{
    F2 s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, add_rn(s.lo, a.lo));
}
CPD_FF_HD F2 mul(F2 a, F2 b)
{
    const float p = mul_rn(a.hi, b.hi);
    const float e = fmaf_(a.hi, b.hi, -p);
    const float lo = fmaf_(a.hi, b.lo, fmaf_(a.lo, b.hi, e));
    return fast_two_sum(p, lo);
}

CPD_FF_HD float u2f(uint32_t v)
{
#if defined(__CUDA_ARCH__)
    return __uint2float_rn(v);
#else
    return (float)v;
#endif
}
CPD_FF_HD int clz64(uint64_t v)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
CPD_FF_HD float ldexp_f(float v, int e)
{
    // v * 2^e for |e| small enough that 2^e is a normal float
    uint32_t b = (uint32_t)(e + 127) << 23;
    float s;
#if defined(__CUDA_ARCH__)
    s = __uint_as_float(b);
#else
    std::memcpy(&s, &b, 4);
#endif
    return v * s;
}

// Table of log2(c_i) and 1/c_i, c_i = 1 + i/256, as float-float pairs:
// entries [4 i .. 4 i + 3] = {log2 hi, log2 lo, inv hi, inv lo}.
constexpr int kLogTable = 256;

// Splits an f64 into a float-float pair.
CPD_FF_HD void split(double v, float &hi, float &lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// Host: fills the 4 * 256 floats of the table.
inline void make_log_table(float *t)
{
    for (int i = 0; i < kLogTable; i++) {
        const double c = 1.0 + i / 256.0;
        split(std::log2(c), t[4 * i], t[4 * i + 1]);
        split(1.0 / c, t[4 * i + 2], t[4 * i + 3]);
    }
}

// An integer c >= 1 (c < 2^64) as a float-float (the top 24 bits exact, the next 24
// rounded): relative error below 2^-47.
CPD_FF_HD F2 from_u64(uint64_t c)
{
    const int lz = clz64(c);
    const int e = 63 - lz;                 // c in [2^e, 2^(e+1))
    if (e < 24) return F2{u2f((uint32_t)c), 0.f};
    const int s = e - 23;                  // drop s low bits for the hi part
    const uint64_t top = c >> s;           // 24 bits
    const uint64_t rest = c - (top << s);  // < 2^s
    const int s2 = s > 24 ? s - 24 : 0;
    const float hi = ldexp_f(u2f((uint32_t)top), s);
    const float lo = ldexp_f(u2f((uint32_t)(rest >> s2)), s2);
    return fast_two_sum(hi, lo);
}

// log2(c) for an integer c >= 1, float-float, absolute error < 1e-12. `tab` is the
// table above (any memory space).
CPD_FF_HD F2 log2_u64(uint64_t c, const float *tab)
{
    const int lz = clz64(c);
    const int e = 63 - lz;
    const uint64_t f = (c << lz) << 1;               // fraction bits of the mantissa 1.f
    const uint32_t i = (uint32_t)(f >> 56);          // table index: top 8 bits
    const uint64_t d = f & ((1ull << 56) - 1);       // remainder: m - c_i = d 2^-64
    // d as float-float in units of 2^-64: top 24 bits exact, next 24 rounded
    const float dh = ldexp_f(u2f((uint32_t)(d >> 32)), 32 - 64);
    const float dl = ldexp_f(u2f((uint32_t)((d >> 8) & 0xffffffu)), 8 - 64);
    const F2 dd = fast_two_sum(dh, dl);
    const F2 inv{tab[4 * i + 2], tab[4 * i + 3]};
    const F2 r = mul(dd, inv);                       // r = (m - c_i)/c_i in [0, 2^-8)
    const F2 k{1.44269502f, 1.92596299e-8f};         // 1/ln 2 as float-float
    const F2 t1 = mul(r, k);                          // r / ln 2
    const F2 t2 = mul(mul(r, r), F2{-0.5f * k.hi, -0.5f * k.lo});  // -r^2 / (2 ln 2)
    // (r^3/3 - r^4/4 + r^5/5) / ln 2 < 2^-24: FP32 suffices
    const float x = r.hi;
    const float t3 = x * x * x * fmaf_(x, fmaf_(x, 0.2f, -0.25f), 0.333333343f) * 1.44269502f;
    F2 s = add(F2{tab[4 * i], tab[4 * i + 1]}, t1);
    s = add(s, t2);
    s = add_f(s, t3);
    return add_f(s, (float)e);
}

}  // namespace ff
}  // namespace cpd
