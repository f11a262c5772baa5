// Double-float arithmetic: a value held as an unevaluated sum hi + lo of two FP32 numbers
// (about 48 significant bits), on GB300's FP32 pipes, whose rate is far above its FP64 rate.
// Algorithms: Knuth's two-sum, Dekker's fast two-sum, the FMA two-product, and the double-float
// add / multiply built from them (as in the QD library of Hida, Li and Bailey).  Conversions
// between FP64 and double-float use integer operations on the bit patterns, not the FP64 unit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#if defined(__CUDACC__)
#define EQC_HD __host__ __device__ __forceinline__
#else
#define EQC_HD inline
#endif

namespace eqc {

struct df {
    float hi, lo;
};

#if defined(__CUDA_ARCH__)
EQC_HD float df_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
EQC_HD float df_add_rn(float a, float b) { return __fadd_rn(a, b); }
EQC_HD float df_sub_rn(float a, float b) { return __fsub_rn(a, b); }
EQC_HD float df_mul_rn(float a, float b) { return __fmul_rn(a, b); }
EQC_HD int64_t df_bits64(double x) { return __double_as_longlong(x); }
EQC_HD double df_from_bits64(int64_t b) { return __longlong_as_double(b); }
EQC_HD float df_from_bits32(int32_t b) { return __int_as_float(b); }
EQC_HD int32_t df_bits32(float x) { return __float_as_int(x); }
#else
EQC_HD float df_fma(float a, float b, float c) { return fmaf(a, b, c); }
EQC_HD float df_add_rn(float a, float b) { volatile float s = a + b; return s; }
EQC_HD float df_sub_rn(float a, float b) { volatile float s = a - b; return s; }
EQC_HD float df_mul_rn(float a, float b) { volatile float s = a * b; return s; }
EQC_HD int64_t df_bits64(double x) { int64_t b; __builtin_memcpy(&b, &x, 8); return b; }
EQC_HD double df_from_bits64(int64_t b) { double x; __builtin_memcpy(&x, &b, 8); return x; }
EQC_HD float df_from_bits32(int32_t b) { float x; __builtin_memcpy(&x, &b, 4); return x; }
EQC_HD int32_t df_bits32(float x) { int32_t b; __builtin_memcpy(&b, &x, 4); return b; }
#endif

// s + e = a + b exactly
EQC_HD void two_sum(float a, float b, float& s, float& e) {
    s = df_add_rn(a, b);
    const float bb = df_sub_rn(s, a);
    e = df_add_rn(df_sub_rn(a, df_sub_rn(s, bb)), df_sub_rn(b, bb));
}
// s + e = a + b exactly, |a| >= |b|
EQC_HD void fast_two_sum(float a, float b, float& s, float& e) {
    s = df_add_rn(a, b);
    e = df_sub_rn(b, df_sub_rn(s, a));
}
EQC_HD df df_add(df x, df y) {
    float s, e;
    two_sum(x.hi, y.hi, s, e);
    e = df_add_rn(e, df_add_rn(x.lo, y.lo));
    df r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
EQC_HD df df_neg(df x) { return df{-x.hi, -x.lo}; }
EQC_HD df df_sub(df x, df y) { return df_add(x, df_neg(y)); }
EQC_HD df df_mul(df x, df y) {
    const float p = df_mul_rn(x.hi, y.hi);
    float e = df_fma(x.hi, y.hi, -p);
    e = df_fma(x.hi, y.lo, e);
    e = df_fma(x.lo, y.hi, e);
    df r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}

// FP64 -> double-float: hi carries the 24 leading significand bits (truncated), lo the next 24
// (rounded); |x| outside [2^-90, 2^120] maps to hi = lo = 0 (far below or above any value the
// stiffness apply sees: displacements, forces).  Integer operations only.
EQC_HD df df_from_double(double x) {
    const int64_t b = df_bits64(x);
    const int32_t e = (int32_t)((b >> 52) & 0x7ff);
    if (e < 1023 - 90 || e > 1023 + 120) return df{0.f, 0.f};
    const int32_t sgn = (int32_t)((uint64_t)b >> 63) << 31;
    const int64_t m = b & 0xfffffffffffffLL;                 // 52 fraction bits
    const float hi = df_from_bits32(sgn | ((e - 1023 + 127) << 23) | (int32_t)(m >> 29));
    const int32_t rem = (int32_t)(m & 0x1fffffff);          // 29 remaining fraction bits
    // lo = +-rem * 2^(e - 1023 - 52): rem as a float (rounded to 24 bits), then the exponent
    const float rf = (float)rem;                             // < 2^29, exact up to rounding
    if (rem == 0) return df{hi, 0.f};
    const int32_t rb = df_bits32(rf);
    const int32_t re = ((rb >> 23) & 0xff) + (e - 1023 - 52);  // biased exponent of lo
    if (re <= 0) return df{hi, 0.f};
    return df{hi, df_from_bits32(sgn | (re << 23) | (rb & 0x7fffff))};
}

// double-float -> FP64 (one FP64 add; the widenings are exact and use integer operations)
EQC_HD double df_widen(float f) {
    const int32_t b = df_bits32(f);
    const int32_t e = (b >> 23) & 0xff;
    if (e == 0) return 0.0;                                   // zero (and FP32 denormals)
    const int64_t sgn = (int64_t)((uint32_t)b >> 31) << 63;
    const int64_t m = (int64_t)(b & 0x7fffff) << 29;
    return df_from_bits64(sgn | ((int64_t)(e - 127 + 1023) << 52) | m);
}
EQC_HD double df_to_double(df x) { return df_widen(x.hi) + df_widen(x.lo); }

#if defined(__CUDACC__)
// x * 2^e (p2 = 2^e), exact: the exponent field moved by integer arithmetic where x and the
// result are normal FP64 numbers, else the FP64 multiply (zeros, subnormals, infinities, NaNs,
// a result out of the normal range).
__device__ __forceinline__ double pow2_scale(double x, int e, double p2) {
    const int64_t b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff), en = ex + e;
    if (ex != 0 && ex != 0x7ff && en > 0 && en < 0x7ff) return __longlong_as_double(b + ((int64_t)e << 52));
    return x * p2;
}
// FP64 -> FP32 through the double-float split (integer operations and one FP32 add) inside
// df_from_double's range [2^-90, 2^120]: the nearest FP32 number but for the rare remainders that
// round to a tie on the way (then one unit in the last place off).  Outside it (zeros, tiny and
// huge values, infinities, NaNs) the hardware conversion, so those propagate as they should.
__device__ __forceinline__ float f64_to_f32(double x) {
    const int e = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
    if (e < 1023 - 90 || e > 1023 + 120) return __double2float_rn(x);
    const df d = df_from_double(x);
    return __fadd_rn(d.hi, d.lo);
}
#endif

}  // namespace eqc
