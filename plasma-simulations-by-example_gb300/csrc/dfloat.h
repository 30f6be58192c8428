/*
 * dfloat.h -- double-float arithmetic shared by the solver and computeEF:
 * a value as an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi) / 2),
 * ~48 significant bits, on the float pipes.  TwoSum (Knuth) and Fast2Sum
 * (Dekker) give the exact rounding error of a sum; a product's error comes
 * from one FMA.  (D. E. Knuth, TAOCP vol. 2, 4.2.2; T. J. Dekker, Numer.
 * Math. 18, 1971.)  The products use explicit FMAs.
 */
#pragma once
#include <cuda_runtime.h>

namespace espic {

struct dfl {
    float h, l;
};
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
    const float s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dfl df_fast2(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ dfl df_add(dfl x, dfl y) {
    const dfl s = df_two_sum(x.h, y.h);
    return df_fast2(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ dfl df_neg(dfl x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dfl df_mul(dfl x, dfl y) {
    const float p = x.h * y.h;
    const float e = __fmaf_rn(x.h, y.h, -p);
    return df_fast2(p, __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, e)));
}
__device__ __forceinline__ dfl df_of(double v) {
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}
/* df_of on the integer pipes: hi = RN_f(v) from the 53-bit significand
 * rounded to 24 bits (ties to even), lo = RN_f(v - hi) from the exact
 * remainder (|r| <= 2^28).  False for magnitudes outside [2^-60, 2^60]
 * (zero included), which the caller converts otherwise. */
__device__ __forceinline__ bool df_split_int(double v, dfl &out) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 60 || e > 1023 + 60) return false;
    const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
    unsigned long long mh = m >> 29;
    const unsigned long long rem = m & 0x1fffffffull;
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (mh & 1))) mh++;
    const int r = (int)((long long)m - (long long)(mh << 29));
    int eh = e - 1023 + 127;
    if (mh == (1ull << 24)) {
        mh >>= 1;
        eh++;
    }
    const unsigned int sgn = (unsigned int)(b >> 32) & 0x80000000u;
    const float hi = __uint_as_float(sgn | ((unsigned int)eh << 23) | ((unsigned int)mh & 0x7fffffu));
    /* r 2^(e - 1075), the power of two built from its exponent bits */
    const float scale = __uint_as_float((unsigned int)(e - 1075 + 127) << 23);
    const float lo = __int2float_rn(r) * scale;
    out = {hi, sgn ? -lo : lo};
    return true;
}
/* df_of(v), on the integer pipes for |v| in [2^-60, 2^60] (the steps of
 * df_split_int) */
__device__ __forceinline__ dfl df_split(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 60 || e > 1023 + 60) return df_of(v);
    const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
    unsigned long long mh = m >> 29;
    const unsigned long long rem = m & 0x1fffffffull;
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (mh & 1))) mh++;
    const int r = (int)((long long)m - (long long)(mh << 29));
    int eh = e - 1023 + 127;
    if (mh == (1ull << 24)) {
        mh >>= 1;
        eh++;
    }
    const unsigned int sgn = (unsigned int)(b >> 32) & 0x80000000u;
    const float hi = __uint_as_float(sgn | ((unsigned int)eh << 23) | ((unsigned int)mh & 0x7fffffu));
    const float scale = __uint_as_float((unsigned int)(e - 1075 + 127) << 23);
    const float lo = __int2float_rn(r) * scale;
    return {hi, sgn ? -lo : lo};
}
__device__ __forceinline__ float2 df_pack(dfl x) { return make_float2(x.h, x.l); }
__device__ __forceinline__ dfl df_unpack(float2 v) { return {v.x, v.y}; }

/* RN_f of a double-float q = (qh, ql) known to lie within `bound` of the
 * float64 value whose float rounding is wanted: qh when q is farther than
 * bound from both float rounding boundaries around qh (the midpoints at
 * qh +- ulp/2); false for a power-of-two qh (its lower midpoint is a quarter
 * ulp away) and for tiny or huge magnitudes, which the caller rounds from
 * the float64 value itself */
__device__ __forceinline__ bool f32_of_df(dfl q, float bound, float &out) {
    const unsigned int eb = __float_as_uint(q.h) & 0x7f800000u;
    if (eb < (30u << 23) || eb > (250u << 23) || (__float_as_uint(q.h) & 0x7fffffu) == 0u) return false;
    const float half_ulp = __uint_as_float(eb - (24u << 23));
    if (!(half_ulp - fabsf(q.l) > bound)) return false;
    out = q.h;
    return true;
}

}  // namespace espic
