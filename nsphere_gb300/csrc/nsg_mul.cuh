// nsg_mul.cuh -- IEEE-754 double multiplication a*b, round to nearest even, computed on
// the integer pipes.
//
// GB300 issues FP64 at 1/64 of its FP32 rate: about 1.6 DMUL results per clock per SM,
// measured, against dozens of 32-bit integer multiply-adds, shifts and logic operations
// (which never issue to the FP64 pipe).  The level-0 and rank-force passes are bound by
// the FP64 pipe, so part of their multiplications run here instead, on the
// integer-multiply (FMA-heavy) and ALU pipes, beside the FP64 operations that stay.
//
// Method (schoolbook): the 53-bit significands split into 32-bit halves give the
// 106-bit product P = hh 2^64 + (hl + lh) 2^32 + ll from four 32 x 32 -> 64-bit
// products; P lies in [2^104, 2^106), its top 53 bits are the significand, the next
// bit rounds, and any bit below sticks.  The exponent is ea + eb - 1023 (+1 when bit
// 105 is set); adding the rounded significand to the shifted exponent lets a rounding
// carry move into the exponent field (and a carry out of the largest exponent give
// infinity, as IEEE rounding does).
// `ok` is false -- and the caller multiplies on the FP64 pipe -- for a zero, subnormal,
// infinite or NaN operand and for a product that leaves the normal range below.
#pragma once
#include "nsg_div.cuh"

namespace nsg {

NSG_HD double mul_rn_int(double a, double b, bool &ok)
{
    const uint64_t ua = div_bits(a), ub = div_bits(b);
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
    const uint64_t sign = (ua ^ ub) & (1ull << 63);
    const uint64_t MANT = (1ull << 52) - 1ull, HID = 1ull << 52;
    const uint64_t ma = (ua & MANT) | HID, mb = (ub & MANT) | HID;
    const uint32_t al = (uint32_t)ma, ah = (uint32_t)(ma >> 32);
    const uint32_t bl = (uint32_t)mb, bh = (uint32_t)(mb >> 32);
    const uint64_t ll = (uint64_t)al * bl;
    const uint64_t mid = (uint64_t)al * bh + (uint64_t)ah * bl;     // < 2^54
    const uint64_t hh = (uint64_t)ah * bh;                           // < 2^42
    const uint64_t plo = ll + (mid << 32);
    const uint64_t phi = hh + (mid >> 32) + (plo < ll ? 1ull : 0ull);   // P = phi 2^64 + plo
    const uint32_t t = (uint32_t)(phi >> 41);                        // bit 105 of P
    uint64_t m = (phi << (12 - t)) | (plo >> (52 + t));               // P >> (52 + t): 53 bits
    const uint64_t rbit = (plo >> (51 + t)) & 1ull;
    const uint64_t sticky = (plo << (13 - t)) != 0ull ? 1ull : 0ull;
    m += rbit & (sticky | (m & 1ull));
    const int32_t e = (int32_t)ea + (int32_t)eb - 1023 + (int32_t)t;  // biased exponent of the result
    ok = (ea - 1u < 2046u) && (eb - 1u < 2046u) && (uint32_t)(e - 1) < 2046u;
    return div_from_bits(sign | (((uint64_t)(uint32_t)(e - 1) << 52) + m));
}

#if defined(__CUDACC__)
// Correctly rounded a * b, bit-identical to __dmul_rn: the integer form, with the FP64
// pipe's multiplication behind a call for the operands it declines (a call cannot be
// if-converted, so the FP64 instruction issues only when it is needed).
// (Operands cross the call as bit patterns, as for div_rn_slow.)
static __device__ __noinline__ double mul_rn_slow(unsigned long long ua, unsigned long long ub)
{
    return __dmul_rn(__longlong_as_double((long long)ua), __longlong_as_double((long long)ub));
}

__device__ __forceinline__ double mul_rn(double a, double b)
{
    bool ok;
    double q = mul_rn_int(a, b, ok);
    if (!ok) q = mul_rn_slow(div_bits(a), div_bits(b));
    return q;
}
#endif

}  // namespace nsg
