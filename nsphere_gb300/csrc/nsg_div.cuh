// nsg_div.cuh -- IEEE-754 double division a/b, round to nearest even, computed on
// the integer and single-precision pipes.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, and a double division on the FP64
// pipe costs about ten FP64 issue slots.  The integrators of the step perform
// several divisions per force evaluation (nsphere.c:513, :535, :575, :599), so
// division throughput bounds the step.  The routines here return the same bits as
// IEEE division (the CPU reference's `/`) for every pair of finite normal operands
// whose quotient is a finite normal number; all other operands (zero, subnormal,
// infinite, NaN, quotient out of the normal range) go to the hardware division.
//
// Two forms:
//   div_rn_lat  three quotient digits from an FP32 reciprocal with exact integer
//               remainders (below).  Few, short steps: the serial chains use it,
//               and so do the throughput kernels (div_rn), once its fallback sits
//               behind a call;
//   div_rn_fast a Newton-Raphson reciprocal in fixed point, then an exactly
//               verified quotient; the division self-test cross-checks it against
//               the hardware and the latency form.
//
// div_rn_fast (a textbook method):
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

// x as a float for x in [2^23, 2^24), from its bits: exponent 23, the low 23 bits
// as the fraction.  Exact, and one logic operation instead of a conversion.
NSG_HD float div_f24(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float((150u << 23) | (x & 0x7fffffu));
#else
    return (float)x;
#endif
}

// Estimate of 2^76 / fb for fb in [2^23, 2^24) as an integer, relative error < 2^-21.
// The estimate y lies in (2^-24, 2^-23], so y 2^76 is an integer of 53 or 54 bits:
// its 24-bit significand shifted left by (biased exponent of y) - 74.  Building it
// from the bits keeps a 64-bit conversion, which shares the FP64 pipe on GB300, out
// of the integer division.
NSG_HD int64_t div_recip_seed(uint32_t mb_top24)
{
#if defined(__CUDA_ARCH__)
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(div_f24(mb_top24)));
    const uint32_t fy = __float_as_uint(y);
    return (int64_t)((fy & 0x7fffffu) | 0x800000u) << ((int)(fy >> 23) - 74);
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
// division about 590; this routine runs on the integer and FP32 pipes, with no
// conversion instruction on its dependent path.
//
// Method (digit recurrence with an approximate reciprocal and exact remainders):
//   A = ma or 2 ma so that A/mb lies in [1, 2);  y ~ 2^29/mb in single precision
//   from rcp.approx of the top 24 bits of mb; s_j = y 2^(k_j + d_j - 29) (exact).
//   Digit j: t = float(r >> k_j), exact; q_j = round(t s_j) ~ r 2^(d_j) / mb;
//   the next remainder r 2^(d_j) - q_j mb.  With (d, k) = (21, 31), (18, 35),
//   (14, 34) from r = A:
//     q1 ~ A 2^21 / mb,  r1 = A 2^21 - q1 mb
//     q2 ~ r1 2^18 / mb, r2 = r1 2^18 - q2 mb
//     q3 ~ r2 2^14 / mb, r3 = r2 2^14 - q3 mb
//   and Q = q1 2^32 + q2 2^14 + q3 satisfies A 2^53 = Q mb + r3 exactly.
//   Conversions use magic numbers: an integer below 2^23 (or of magnitude below
//   2^22) placed in the fraction of 2^23 (1.5 2^23) minus that constant is the
//   integer as a float, exactly; fma(t, s, 2^23) (1.5 2^23) rounds t s to the
//   nearest integer in one rounding, read back from the fraction bits.
// Error bounds.  With the estimate's relative error e (truncation of mb to 24
// bits and rcp.approx: below 2^-22; below 10 2^-23 for the host tests that
// perturb it by 8 ulps), digit j misses its ideal value by at most
//   1/2 + 2^(k_j + d_j - 52) + |r| 2^(d_j) e / mb:
//   digit 1 by 11.5 at most, so |r1| < 11.5 mb < 2^56.6 and |r1 >> 35| < 2^22;
//   digit 2 by 1/2 + 2 + 11.5 2^18 e < 6.1, so |r2| < 2^55.7 and |r2 >> 34| < 2^22;
//   digit 3 by 1/2 + 2^-4 + 6.1 2^14 e < 0.69, so |r3| < mb.
// Every remainder is far below 2^63, so its value modulo 2^64 is exact, and one
// step (r3 < 0: Q - 1, r3 + mb) makes Q the floor and 0 <= r3 < mb the exact
// remainder: round bit Q & 1, sticky r3 != 0.
// There are no branches: every operand runs the same instructions, and `ok` says
// whether the result stands (both operands normal, or a +-0 dividend over a normal
// divisor, and a normal quotient); otherwise the caller divides in hardware.  A
// branch to a fallback inside the chain costs more than the division itself, so
// callers accumulate the flags and redo the whole chain when one is set.
NSG_HD float div_lat_rcp(int32_t x)
{
#if defined(__CUDA_ARCH__)
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(div_f24((uint32_t)x)));   // x in [2^23, 2^24)
    return y;
#elif defined(NSG_DIV_HOST_RCP)
    return NSG_DIV_HOST_RCP(x);   // host tests substitute perturbed estimates
#else
    return 1.0f / (float)x;
#endif
}

NSG_HD float div_fbits(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}

NSG_HD uint32_t div_ubits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}

NSG_HD float div_fsub(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

NSG_HD float div_ffma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}

// First digit: t = x for 0 <= x < 2^23; round(t s) for 0 <= t s < 2^23 - 1/2.
NSG_HD uint32_t div_lat_digit_u(uint32_t x, float s)
{
    const float t = div_fsub(div_fbits(0x4B000000u | x), 8388608.0f);
    return div_ubits(div_ffma(t, s, 8388608.0f)) - 0x4B000000u;
}

// Later digits: t = x for |x| < 2^22; round(t s) for |t s| < 2^22 - 1/2.
NSG_HD int32_t div_lat_digit_s(int32_t x, float s)
{
    const float t = div_fsub(div_fbits(0x4B400000u + (uint32_t)x), 12582912.0f);
    return (int32_t)(div_ubits(div_ffma(t, s, 12582912.0f)) - 0x4B400000u);
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
    const float y = div_lat_rcp((int32_t)(mb >> 29));
    const uint32_t q1 = div_lat_digit_u((uint32_t)(A >> 31), y * 0x1p23f);
    const int64_t r1 = (int64_t)((A << 21) - (uint64_t)q1 * mb);
    const int32_t q2 = div_lat_digit_s((int32_t)(r1 >> 35), y * 0x1p24f);
    const int64_t r2 = (int64_t)(((uint64_t)r1 << 18) - (uint64_t)(int64_t)q2 * mb);
    const int32_t q3 = div_lat_digit_s((int32_t)(r2 >> 34), y * 0x1p19f);
    const int64_t r3 = (int64_t)(((uint64_t)r2 << 14) - (uint64_t)(int64_t)q3 * mb);
    const int64_t Q = ((int64_t)q1 << 32) + ((int64_t)q2 << 14) + (int64_t)q3;
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
// The FP64 pipe's division behind a call: the compiler cannot predicate or hoist the
// division's instructions into the caller, so they run only for the operands the
// integer forms leave (a predicated inline fallback halves the throughput).  The
// operands cross the call as bit patterns: passed as doubles, the call costs the caller
// one FP64-pipe instruction on every division, taken or not (measured with the pipe
// counters), which the throughput kernels, bound by that pipe, cannot spare.
static __device__ __noinline__ double div_rn_slow(unsigned long long ua, unsigned long long ub)
{
    return __ddiv_rn(__longlong_as_double((long long)ua), __longlong_as_double((long long)ub));
}

// Correctly rounded a / b (round to nearest even), bit-identical to __ddiv_rn: the
// latency form, whose few integer and FP32 steps also give the highest throughput
// once its fallback sits behind a call (248 G/s alone against 110 for div_rn_fast).
__device__ __forceinline__ double div_rn(double a, double b)
{
    bool ok;
    double q = div_rn_lat(a, b, ok);
    if (!ok) q = div_rn_slow(div_bits(a), div_bits(b));
    return q;
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
