// Double-float arithmetic shared by the kernels of libopencmp_gpu.so (sm_103a): values are
// unevaluated sums hi + lo of two floats (about 48 significant bits), products carry an FMA-exact
// error term, sums an exact TwoSum of the high parts. Floats are widened to doubles with integer
// operations (exact for normal numbers; subnormal floats, below 1.2e-38, are flushed to zero).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ocmp {

__device__ __forceinline__ void ff_add(float& sh, float& sl, float ph, float pl) {
    const float s = __fadd_rn(sh, ph);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
    sl = __fadd_rn(__fadd_rn(sl, pl), err);
    sh = s;
}
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float& ph, float& pl) {
    ph = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -ph);
    e = __fmaf_rn(ah, bl, e);
    pl = __fmaf_rn(al, bh, e);
}
__device__ __forceinline__ double f2d_exact(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(b & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)sgn);
    if (e == 0xffu) return (double)f;
    const unsigned long long d = sgn | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)d);
}
__device__ __forceinline__ double ff_to_double(float h, float l) { return f2d_exact(h) + f2d_exact(l); }
__device__ __forceinline__ float2 ff_split(double x) {
    const float h = __double2float_rn(x);
    return make_float2(h, __double2float_rn(x - f2d_exact(h)));
}

// (ah + al)(bh + bl), renormalised so the pair can feed further products
__device__ __forceinline__ float2 ff_prod(float2 a, float2 b) {
    float ph, pl;
    ff_mul(a.x, a.y, b.x, b.y, ph, pl);
    const float s = __fadd_rn(ph, pl);
    return make_float2(s, __fsub_rn(pl, __fsub_rn(s, ph)));
}

// x = hi + lo exactly up to the I2F rounding of the low 29 mantissa bits (relative error below 2^-47);
// |x| below 2^-74 keeps only hi, infinities and NaN pass through in hi
__device__ __forceinline__ float2 split_d(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    if (e == 0x7ffu || e < 897u) return make_float2((float)x, 0.f);  // non-finite, or below FP32's normal range
    const float hi = __uint_as_float(sgn | ((e - 896u) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
    const unsigned rem = (unsigned)(b & 0x1fffffffu);
    if (rem == 0u || e < 949u) return make_float2(hi, 0.f);
    // rem * 2^(e - 1075), sign of x; the power of two is a normal float for e >= 949
    const float lo = __int2float_rn((int)rem) * __uint_as_float((e - 948u) << 23);
    return make_float2(hi, sgn ? -lo : lo);
}

// (a.x + a.y) + s (b.x + b.y) for s = +1 / -1, renormalised so |lo| <= ulp(hi) / 2
__device__ __forceinline__ float2 ff_addn(float2 a, float2 b, bool neg) {
    float h = a.x, l = a.y;
    ff_add(h, l, neg ? -b.x : b.x, neg ? -b.y : b.y);
    const float s = __fadd_rn(h, l);
    return make_float2(s, __fsub_rn(l, __fsub_rn(s, h)));
}

}  // namespace ocmp
