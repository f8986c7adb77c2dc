// nsg_div.cuh -- IEEE-754 double division a/b, round to nearest even, computed on
// the integer and single-precision pipes.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, and a double division on the FP64
// pipe costs about ten FP64 issue slots.  The integrators of the step perform
// several divisions per force evaluation (nsphere.c:513, :535, :575, :599), so
// division throughput bounds the step.  This routine returns the same bits as
// IEEE division (the CPU reference's `/`) for every pair of finite normal operands
// whose quotient is a finite normal number; all other operands (zero, subnormal,
// infinite, NaN, quotient out of the normal range) go to the hardware division.
//
// Method (a textbook Newton-Raphson reciprocal in fixed point, then an exactly
// verified quotient):
//   mantissas ma, mb in [2^52, 2^53); A = ma or 2 ma so that A/mb lies in [1, 2);
//   R ~ 2^105/mb: single-precision reciprocal estimate (rel. error < 2^-21),
//       then two Newton steps R += R (2^105 - mb R) / 2^105 in 64/128-bit integers;
//   Q ~ floor(A 2^53 / mb) from A R / 2^52, refined once by the exact remainder
//       rem = A 2^53 - Q mb (computed mod 2^64; its true value fits in 63 bits),
//       then stepped until 0 <= rem < mb, which makes Q the exact floor;
//   Q carries 53 mantissa bits plus the round bit; rem != 0 is the sticky bit.
// Any estimate outside the stepping range falls back to the hardware division,
// so an error in the estimate costs time, never correctness.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define NSG_HD __host__ __device__ __forceinline__
#else
#define NSG_HD static inline
#endif

namespace nsg {

NSG_HD uint64_t div_umulhi(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

NSG_HD int64_t div_mulhi(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return (int64_t)(((__int128)a * b) >> 64);
#endif
}

NSG_HD uint64_t div_bits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    __builtin_memcpy(&u, &x, 8);
    return u;
#endif
}

NSG_HD double div_from_bits(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    __builtin_memcpy(&x, &u, 8);
    return x;
#endif
}

// Estimate of 2^76 / fb for fb in [2^23, 2^24) as an integer, relative error < 2^-21.
NSG_HD int64_t div_recip_seed(uint32_t mb_top24)
{
#if defined(__CUDA_ARCH__)
    float fb = (float)mb_top24;  // exact: fewer than 25 significant bits
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(fb));
    return (int64_t)__float2ll_rz(y * 0x1p76f);
#else
    float fb = (float)mb_top24;
    float y = 1.0f / fb;
    return (int64_t)(y * 0x1p76f);
#endif
}

// Fast path; returns false when the operands or the quotient leave the normal range
// or an estimate misses (the caller then uses the hardware division).
NSG_HD bool div_rn_fast(double a, double b, double *out)
{
    const uint64_t ua = div_bits(a), ub = div_bits(b);
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
    if (eb - 1u < 2046u && (ua << 1) == 0ull) {              // +-0 / normal: signed zero
        *out = div_from_bits((ua ^ ub) & (1ull << 63));
        return true;
    }
    if (ea - 1u >= 2046u || eb - 1u >= 2046u) return false;  // zero, subnormal, inf, NaN
    const uint64_t MANT = (1ull << 52) - 1ull, HID = 1ull << 52;
    const uint64_t ma = (ua & MANT) | HID, mb = (ub & MANT) | HID;
    int32_t e = (int32_t)ea - (int32_t)eb + 1023;
    uint64_t A = ma;
    if (ma < mb) { A = ma << 1; e -= 1; }
    if ((uint32_t)(e - 1) >= 2046u) return false;            // quotient not a normal number

    // R ~ 2^105 / mb
    int64_t R = div_recip_seed((uint32_t)(mb >> 29));
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const uint64_t plo = mb * (uint64_t)R;
        const uint64_t phi = div_umulhi(mb, (uint64_t)R);
        const uint64_t dlo = 0ull - plo;                     // D = 2^105 - (phi:plo)
        const int64_t dhi = (int64_t)((1ull << 41) - phi - (plo != 0ull ? 1ull : 0ull));
        const int64_t Ds = (int64_t)((uint64_t)dhi << 23) | (int64_t)(dlo >> 41);  // floor(D / 2^41)
        R += div_mulhi(R, Ds);                               // R + floor(R D / 2^105)
    }
    // Q ~ floor(A * 2^53 / mb) = A R / 2^52
    uint64_t Q = div_umulhi(A << 10, (uint64_t)R << 2);
    int64_t rem = (int64_t)((A << 53) - Q * mb);             // exact: |rem| < 2^63
    if (rem >= (int64_t)1 << 59 || rem <= -((int64_t)1 << 59)) return false;
    const int64_t d = div_mulhi(rem << 4, (int64_t)R << 1) >> 46;  // floor(rem R / 2^105) ~ rem / mb
    Q += (uint64_t)d;
    rem -= d * (int64_t)mb;
#pragma unroll
    for (int it = 0; it < 2; it++) {
        if (rem < 0) { Q -= 1; rem += (int64_t)mb; }
        else if (rem >= (int64_t)mb) { Q += 1; rem -= (int64_t)mb; }
    }
    if (rem < 0 || rem >= (int64_t)mb) return false;
    // Q in [2^53, 2^54): 53 mantissa bits and the round bit; rem != 0 is sticky
    uint64_t m = Q >> 1;
    const uint64_t rb = Q & 1ull;
    if (rb && (rem != 0 || (m & 1ull))) m += 1;
    if (m == (1ull << 53)) { m >>= 1; e += 1; if (e > 2046) return false; }
    *out = div_from_bits(((ua ^ ub) & (1ull << 63)) | ((uint64_t)e << 52) | (m & MANT));
    return true;
}

// ---------------------------------------------------------------------------
// Latency-oriented division for serial chains (one particle's Levi-Civita
// substeps).  On GB300 a dependent FP64 operation takes 64 cycles and the FP64
// division about 590; this routine takes about 220 on the integer and FP32 pipes.
//
// Method (digit recurrence with an approximate reciprocal and exact remainders):
//   A = ma or 2 ma so that A/mb lies in [1, 2);  ys ~ 2^48/mb in single precision
//   from rcp.approx of the top 24 bits of mb (relative error < 2^-21);
//   q1 = round(float(A >> 26) ys)            ~ A 2^22 / mb,  r1 = A 2^22 - q1 mb
//   q2 = round(float(r1 >> 28) 4 ys)         ~ r1 2^22 / mb, r2 = r1 2^22 - q2 mb
//   q3 = round(float(r2 >> 28) 2^-11 ys)     ~ r2 2^9 / mb,  r3 = r2 2^9 - q3 mb
//   Q = q1 2^31 + q2 2^9 + q3 satisfies A 2^53 = Q mb + r3 exactly.  Each
//   remainder is computed modulo 2^64; its true value is below 2^58 in magnitude
//   (each digit is within a few units of its ideal value), so the modular result
//   is exact.  |r3| < mb/2, so one step (r3 < 0: Q - 1, r3 + mb) makes Q the floor
//   and 0 <= r3 < mb the exact remainder: round bit Q & 1, sticky r3 != 0.
// There are no branches: every operand runs the same instructions, and `ok` says
// whether the result stands (both operands normal, or a +-0 dividend over a normal
// divisor, and a normal quotient); otherwise the caller divides in hardware.  A
// branch to a fallback inside the chain costs more than the division itself, so
// callers accumulate the flags and redo the whole chain when one is set.
NSG_HD float div_lat_rcp(int32_t x)
{
#if defined(__CUDA_ARCH__)
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(__int2float_rn(x)));
    return y;
#elif defined(NSG_DIV_HOST_RCP)
    return NSG_DIV_HOST_RCP(x);   // host tests substitute perturbed estimates
#else
    return 1.0f / (float)x;
#endif
}

NSG_HD int32_t div_lat_digit(int32_t top, float scale)
{
#if defined(__CUDA_ARCH__)
    return __float2int_rn(__int2float_rn(top) * scale);
#else
    return (int32_t)__builtin_nearbyintf((float)top * scale);
#endif
}

NSG_HD double div_rn_lat(double a, double b, bool &ok)
{
    const uint64_t ua = div_bits(a), ub = div_bits(b);
    const uint32_t ea = (uint32_t)(ua >> 52) & 0x7ffu, eb = (uint32_t)(ub >> 52) & 0x7ffu;
    const uint64_t sign = (ua ^ ub) & (1ull << 63);
    const bool bnorm = eb - 1u < 2046u;
    const bool zero = bnorm && (ua << 1) == 0ull;
    const uint64_t MANT = (1ull << 52) - 1ull, HID = 1ull << 52;
    const uint64_t ma = (ua & MANT) | HID, mb = (ub & MANT) | HID;
    const bool lt = ma < mb;
    const uint64_t A = lt ? ma << 1 : ma;
    const int32_t e = (int32_t)ea - (int32_t)eb + 1023 - (lt ? 1 : 0);
    const float ys = div_lat_rcp((int32_t)(mb >> 29)) * 0x1p19f;
    const int32_t q1 = div_lat_digit((int32_t)(A >> 26), ys);
    const int64_t r1 = (int64_t)((A << 22) - (uint64_t)(int64_t)q1 * mb);
    const int32_t q2 = div_lat_digit((int32_t)(r1 >> 28), ys * 4.0f);
    const int64_t r2 = (int64_t)(((uint64_t)r1 << 22) - (uint64_t)(int64_t)q2 * mb);
    const int32_t q3 = div_lat_digit((int32_t)(r2 >> 28), ys * 0x1p-11f);
    const int64_t r3 = (int64_t)(((uint64_t)r2 << 9) - (uint64_t)(int64_t)q3 * mb);
    const int64_t Q = ((int64_t)q1 << 31) + ((int64_t)q2 << 9) + (int64_t)q3;
    const bool neg = r3 < 0;
    const int64_t rr = neg ? r3 + (int64_t)mb : r3;
    const uint64_t Qc = (uint64_t)(neg ? Q - 1 : Q);
    uint64_t m = Qc >> 1;
    m += (Qc & 1ull) & ((uint64_t)(rr != 0) | (m & 1ull));
    // m in [2^52, 2^53]; 2^53 carries into the exponent field
    const uint64_t bits = sign | (((uint64_t)(uint32_t)(e - 1) << 52) + m);
    ok = zero || ((ea - 1u < 2046u) && bnorm && ((uint32_t)(e - 1) < 2045u) && rr >= 0 && rr < (int64_t)mb);
    return div_from_bits(zero ? sign : bits);
}

#if defined(__CUDACC__)
// Correctly rounded a / b (round to nearest even), bit-identical to __ddiv_rn.
__device__ __forceinline__ double div_rn(double a, double b)
{
    double q;
    if (div_rn_fast(a, b, &q)) return q;
    return __ddiv_rn(a, b);
}

// The FP64 pipe's division with the +-0 / normal case answered directly (IEEE:
// a zero with the sign a XOR b).  The innermost particle has a zero gravity
// numerator, so its serial chains divide zero in every force evaluation.
__device__ __forceinline__ double div_rn_hw(double a, double b)
{
    const uint64_t ua = div_bits(a), ub = div_bits(b);
    const uint32_t eb = (uint32_t)(ub >> 52) & 0x7ffu;
    if (eb - 1u < 2046u && (ua << 1) == 0ull) return div_from_bits((ua ^ ub) & (1ull << 63));
    return __ddiv_rn(a, b);
}
#endif

}  // namespace nsg
