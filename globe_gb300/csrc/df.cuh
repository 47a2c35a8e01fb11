// df.cuh -- double-float arithmetic for the record kernels of the mixed-precision solve.
//
// A value is the unevaluated sum h + l of two FP32 numbers with |l| <= ulp(h)/2, about 48
// significant bits.  GB300's FP32 pipe is many times its FP64 pipe, and the record-level
// vector updates of block PCG are a few multiply-adds per record and column, so under
// GLOBE_PREC_MIXED they run in these pairs (stored as float2 in the 8 bytes of a double).
//
// The error-free transformations are the published ones: Knuth's two-sum, Dekker's fast
// two-sum and the FMA form of Dekker's exact product (Dekker 1971; Knuth, TAOCP vol. 2,
// 4.2.2; Hida, Li and Bailey, "Library for double-double and quad-double arithmetic", 2001).
// add() is the "sloppy" double-double sum: its error is within a few units of 2^-48 of
// |a| + |b|, which is what the vector updates need (FP64 gives 2^-53 of the result).
// Every FP32 operation is an explicit round-to-nearest intrinsic, so the compiler neither
// contracts nor reorders them.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

namespace globe {
namespace df {

struct D {
    float h, l;
};

__host__ __device__ __forceinline__ D make(float h, float l) {
    D r;
    r.h = h;
    r.l = l;
    return r;
}
__device__ __forceinline__ D zero() { return make(0.0f, 0.0f); }
__device__ __forceinline__ D load(const float2* p) {
    const float2 v = *p;
    return make(v.x, v.y);
}
__device__ __forceinline__ void store(float2* p, D a) { *p = make_float2(a.h, a.l); }

// Conversions.  GB300's FP64 pipe also runs the FP64 <-> FP32 conversion instructions, so
// the per-element ones below work on the bits with integer and FP32 instructions.

// nearest FP32 h, then the nearest FP32 to the remainder (FP64 instructions; for scalars and
// the rare values the bit routes leave to it)
__device__ __forceinline__ D from_double(double d) {
    const float h = __double2float_rn(d);
    return make(h, __double2float_rn(d - (double)h));
}
inline D from_double_host(double d) {
    const float h = (float)d;
    return make(h, (float)(d - (double)h));
}

// d 2^sh as a pair from the bits of d: hi = d 2^sh cut to 24 significant bits, lo = the other
// 29 bits of the significand rounded to 24, so hi + lo is within 2^-47 |d 2^sh|.  Zeros take
// the bit route too; results outside [2^-70, 2^100) in magnitude, subnormals, infinities and
// NaN go through from_double(ldexp(d, sh)).
__device__ __forceinline__ D from_double_scaled(double d, int sh) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(u >> 63) << 31;
    if ((u << 1) == 0ull) return make(__uint_as_float(sign), 0.0f);
    const int E = (int)((u >> 52) & 0x7ffu);
    const int e = E - 1023 + sh;   // exponent of d 2^sh
    if (E == 0 || E == 0x7ff || e < -70 || e >= 100) return from_double(ldexp(d, sh));
    const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((u >> 29) & 0x7fffffu));
    // the low 29 bits times 2^(e - 52), the power of two built from its biased exponent e + 75
    const float lo =
        __fmul_rn(__uint2float_rn((unsigned)(u & 0x1fffffffu)), __uint_as_float((unsigned)(e + 75) << 23));
    return make(hi, sign ? -lo : lo);
}

// FP32 -> FP64 from the bits for zeros and normal numbers (exact); subnormals, infinities and
// NaN through the conversion instruction
__device__ __forceinline__ double f2d(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    const unsigned long long s = (unsigned long long)(b >> 31) << 63;
    if ((b << 1) == 0u) return __longlong_as_double((long long)s);
    if (e == 0u || e == 0xffu) return (double)f;
    return __longlong_as_double(
        (long long)(s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(b & 0x7fffffu) << 29)));
}
// h + l rounded to FP64 (one FP64 instruction)
__device__ __forceinline__ double to_double(D a) { return f2d(a.h) + f2d(a.l); }

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ D two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bv = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
    return make(s, e);
}
// s + e = a + b exactly when |a| >= |b| or a = 0 (Dekker)
__device__ __forceinline__ D fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return make(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ D add(D a, D b) {
    const D s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ D neg(D a) { return make(-a.h, -a.l); }
__device__ __forceinline__ D sub(D a, D b) { return add(a, neg(b)); }
// a.h b.h exactly as p + e by one FMA, plus the cross terms
__device__ __forceinline__ D mul(D a, D b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}
// a b + c
__device__ __forceinline__ D madd(D a, D b, D c) { return add(mul(a, b), c); }

// butterfly sum over the warp (add is commutative, so every lane ends with the same value)
__device__ __forceinline__ D warp_sum(D v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const D w = make(__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o));
        v = add(v, w);
    }
    return v;
}

}  // namespace df

// Per-column power-of-two scaling of a double-float solve: column c runs on s_c b_c with
// s_c = 2^-e, |b_c| = m 2^e, m in [0.5, 1), so its values sit near 1 whatever the scale of the
// data.  col_unscale returns 2^e (1 for a zero or non-finite norm); scaling by powers of two
// is exact, and sqrt(rr) 2^e = sqrt(rr 4^e), so the stopping rule sees the unscaled norms.
__host__ __device__ __forceinline__ int col_scale_exp(double bb) {
    if (!(bb > 0.0) || !(bb <= 1.7976931348623157e308)) return 0;
    int e;
    frexp(sqrt(bb), &e);
    return e;
}
__host__ __device__ __forceinline__ double col_unscale(double bb) { return ldexp(1.0, col_scale_exp(bb)); }

}  // namespace globe
