// usct_convert.cuh -- exact FP64 <-> FP32 conversions in integer arithmetic.
//
// IEEE round to nearest even, the results of the hardware conversions; the
// hardware conversions issue to the FP64 pipe, of which GB300 has very little
// (the TFM kernels were limited by it).
// Zeros and the normal range take the integer path; subnormal, out-of-range,
// infinite and NaN values the hardware one.
#pragma once

#include <cuda_runtime.h>

namespace usct_cvt {

__device__ __forceinline__ float f64_to_f32(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff);
    if (e >= 897 && e <= 1150) {   // FP32 exponent e - 896 in [1, 254]
        const unsigned long long m = b & 0xfffffffffffffULL;
        unsigned r = ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29);
        const unsigned rem = (unsigned)(m & 0x1fffffffULL);   // the 29 dropped bits
        r += (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ? 1u : 0u;
        return __uint_as_float(r | sign);   // a carry into the exponent is exact (to inf at the top)
    }
    if ((b << 1) == 0) return __uint_as_float(sign);
    return __double2float_rn(x);
}

// exact (every FP32 value is an FP64 value)
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u < 254u) {
        const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                                     ((unsigned long long)(e + 896u) << 52) |
                                     ((unsigned long long)(u & 0x7fffffu) << 29);
        return __longlong_as_double((long long)b);
    }
    if ((u << 1) == 0) return __longlong_as_double((long long)((unsigned long long)u << 32));
    return (double)f;
}

}  // namespace usct_cvt
