// Float-float (double-word) arithmetic and the integer-pipe conversions
// between double and pairs of floats.  GB300 issues FP64 at 1/57 of the
// FP32 rate, so kernels that only need ~48 significant bits, or FP32 values
// of FP64 data, work on hi + lo pairs of floats with error-free
// transformations: Knuth's TwoSum, Dekker's Fast2Sum and the FMA product
// error (a*b - p exactly = fmaf(a, b, -p)).
#pragma once

namespace stzg {

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_fast2sum(float a, float b) {
    const float s = a + b;
    return ff{s, b - (s - a)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const float s = a.hi + b.hi, bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    return ff_fast2sum(s, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return ff_fast2sum(p, e);
}
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    const float s = a.hi + b, bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b - bb);
    e += a.lo;
    return ff_fast2sum(s, e);
}

// double -> hi + lo on the integer pipe: hi keeps the sign, the exponent and
// the leading 24 significant bits, lo the remaining 29 bits rounded to a
// float.  |d| below 2^-126 gives 0; below 2^-74 lo is dropped (an absolute
// error under 2^-98).  NaN and infinity pass through in hi.
__device__ __forceinline__ void ff_split_d(double d, float &hi, float &lo) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(u >> 63) << 31;
    const int ex = (int)((u >> 52) & 0x7ff);
    const int ef = ex - 1023 + 127;
    lo = 0.f;
    if (ex == 0x7ff) {
        hi = (u & 0xfffffffffffffull) ? __uint_as_float(0x7fc00000u) : __uint_as_float(sign | 0x7f800000u);
        return;
    }
    if (ef <= 0) {
        hi = __uint_as_float(sign);
        return;
    }
    if (ef >= 255) {
        hi = __uint_as_float(sign | 0x7f800000u);
        return;
    }
    hi = __uint_as_float(sign | ((unsigned)ef << 23) | (unsigned)((u >> 29) & 0x7fffffu));
    const int es = ex - 1075 + 127;  // float exponent field of 2^(ex - 1075)
    if (es > 0) {
        const float r = __uint2float_rn((unsigned)(u & 0x1fffffffu)) * __uint_as_float((unsigned)es << 23);
        lo = sign ? -r : r;
    }
}

// float -> double bits on the integer pipe (exact for normal floats; zero
// and subnormal floats give a signed zero, infinity and NaN keep their class
// and payload).
__device__ __forceinline__ unsigned long long ff_f2d_bits(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xff;
    const unsigned long long man = (unsigned long long)(u & 0x7fffffu) << 29;
    unsigned long long r = (unsigned long long)(u >> 31) << 63;
    if (e == 255) r |= 0x7ff0000000000000ull | man;
    else if (e != 0) r |= ((unsigned long long)(e + 896) << 52) | man;
    return r;
}
__device__ __forceinline__ double ff_f2d(float f) { return __longlong_as_double((long long)ff_f2d_bits(f)); }

// hi + lo as one double without an FP64 instruction, for a pair whose lo is
// at most one 24-bit ulp of hi with lo's sign or half of it with either sign
// (ff_fast2sum and ff_split_d leave them so): lo is counted in units of hi's
// 53-bit ulp (the bits below are dropped, an error below 2^-52 |hi|) and
// added to hi's bit pattern, which stays in hi's binade except where hi is a
// power of two and lo of the other sign (then the units are halved).  Pairs
// with a larger lo take one FP64 addition.
__device__ __forceinline__ double ff_to_d(float hi, float lo) {
    const unsigned uh = __float_as_uint(hi), ul = __float_as_uint(lo);
    const int eh = (uh >> 23) & 0xff, el = (ul >> 23) & 0xff;
    unsigned long long H = ff_f2d_bits(hi);
    if (eh == 0 || eh == 255 || el == 0) return __longlong_as_double((long long)H);
    const int k = eh - el - 29;  // lo = ML * 2^-k units of hi's 53-bit ulp
    if (k < -5) return __longlong_as_double((long long)H) + ff_f2d(lo);
    if (k >= 24) return __longlong_as_double((long long)H);
    const unsigned ml = (1u << 23) | (ul & 0x7fffffu);
    unsigned long long x = k >= 0 ? (unsigned long long)(ml >> k) : (unsigned long long)ml << (-k);
    if ((uh ^ ul) >> 31) {
        if ((H & 0xfffffffffffffull) == 0) x <<= 1;
        H -= x;
    } else {
        H += x;
    }
    return __longlong_as_double((long long)H);
}

// a - b for a = ah + al, b = bh + bl (pairs from ff_split_d), rounded to a
// float: the difference of the high parts by TwoSum (exact) plus the
// difference of the low parts, so the result carries the float rounding of
// a - b itself however close a and b are (~2^-24 relative to |a - b|, plus
// ~2^-48 of |a| and |b| from the split).
__device__ __forceinline__ float ff_diff(float ah, float al, float bh, float bl) {
    const float s = ah - bh, bb = s - ah;
    const float e = (ah - (s - bb)) + (-bh - bb);
    return s + (e + (al - bl));
}

// Leading 24 bits of a double as a float (sign, exponent and truncated
// significand), on the integer pipe: relative error below 2^-23.
__device__ __forceinline__ float ff_hi(double d) {
    float h, l;
    ff_split_d(d, h, l);
    return h;
}

}  // namespace stzg
