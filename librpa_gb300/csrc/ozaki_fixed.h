// Integer arithmetic of the tensor-core Cholesky (k_chol_ozaki.cu), shared by the kernels and
// by a host-compiled unit test.
//
// A row of the panel is scaled by 2^-e (e from its largest magnitude, so every scaled entry v
// lies in (-1, 1)) and cut into OZ_SLICES signed 7-bit digits of |v| 2^56:
//     v = sum_p s_p 2^{-7(p+1)},  s_p in [-127, 127].
// A product of two rows is then 2^{e_i + e_j} sum_d T_d 2^{-7(d+2)}, T_d the integer sum of the
// slice products with p + q = d (d = 0..7).  The groups are combined into the 64-bit
// fixed-point W ~ U / 2^7 with U = sum_d T_d 2^{7(7-d)} (value U 2^{e_i + e_j - 63}), and W is
// turned into a double by integer operations.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define OZ_HD __host__ __device__ __forceinline__
#else
#define OZ_HD inline
#endif

namespace gb {
namespace ozaki {

constexpr int OZ_SLICES = 8;

OZ_HD int clz64(unsigned long long x)
{
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(x));
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

OZ_HD double bits_to_double(unsigned long long b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(b));
#else
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
#endif
}

// Exponent e of a row whose largest magnitude has the FP64 bit pattern mbits (sign cleared):
// max < 2^e; 0 for an all-zero (or subnormal) row.
OZ_HD int row_exponent(unsigned long long mbits)
{
    const int mexp = static_cast<int>(mbits >> 52);
    return mexp ? mexp - 1022 : 0;
}

// The signed 7-bit digits of one entry (FP64 bit pattern u) of a row with exponent e:
// s_p = sign(x) * ((|x| 2^{56-e} truncated) >> (49 - 7 p)) & 127.  Subnormal entries and
// all-zero rows give zero digits.
OZ_HD void slice_digits(unsigned long long u, int e, bool row_nonzero, int (&dig)[OZ_SLICES])
{
    const int bexp = static_cast<int>((u >> 52) & 0x7FF);
    const bool neg = (u >> 63) != 0;
    unsigned long long F = 0;  // |x| 2^(56 - e), truncated
    if (bexp != 0 && row_nonzero)
    {
        const unsigned long long mant = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        const int sh = (bexp - 1023) + 4 - e;  // |x| = mant 2^(bexp - 1075); <= 3 since |x| < 2^e
        F = sh >= 0 ? mant << sh : (sh > -64 ? mant >> (-sh) : 0ull);
    }
    for (int p = 0; p < OZ_SLICES; ++p)
    {
        const int d = static_cast<int>((F >> (49 - 7 * p)) & 127ull);
        dig[p] = neg ? -d : d;
    }
}

// W = round(U / 2^7), U = sum_d T_d 2^{7(7-d)}, from the group sums paired as
// U_g = T_{2g} 2^7 + T_{2g+1} (|T_d| < 2^23, so |U_g| < 2^31).  Exact in 64 bits when the
// true |U| < 2^69 (entries |v| < 1 over K = 64 terms).
OZ_HD long long combine_groups(int u0, int u1, int u2, int u3)
{
    const long long hi = (static_cast<long long>(u0) << 14) + u1;
    const long long lo = (static_cast<long long>(u2) << 14) + u3;
    return (hi << 21) + ((lo + 64) >> 7);
}

// value = w 2^e0 for |w| < 2^63, rounded to nearest (ties away from zero), by integer
// operations only (GB300's FP64 pipe is the scarce unit in the kernels).
OZ_HD double fixed_to_double(long long w, int e0)
{
    if (w == 0) return 0.0;
    const unsigned long long sign = static_cast<unsigned long long>(w) & 0x8000000000000000ull;
    const unsigned long long mag = w < 0 ? 0ull - static_cast<unsigned long long>(w) : static_cast<unsigned long long>(w);
    const int lz = clz64(mag);
    const unsigned long long norm = mag << lz;                       // leading one at bit 63
    unsigned long long mant = (norm >> 11) + ((norm >> 10) & 1ull);  // 53 bits, rounded
    int be = 63 - lz + e0 + 1023;
    if (mant >> 53)
    {
        mant >>= 1;
        ++be;
    }
    if (be <= 0) return 0.0;  // below the normal range: negligible next to the FP64 entries
    return bits_to_double(sign | (static_cast<unsigned long long>(be) << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

} // namespace ozaki
} // namespace gb
