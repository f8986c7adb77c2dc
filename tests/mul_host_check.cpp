// Host check of mul_rn_int (nsg_mul.cuh) against the CPU's IEEE multiplication:
// every operand pair whose product the routine claims must give the same bits.
// Operand classes: random significands and exponents, products near the top and the
// bottom of the normal range, significands with many trailing zeros (exact products
// and exact ties), all-ones significands, powers of two, and signed zeros,
// subnormals, infinities and NaNs (which it must decline).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "nsg_mul.cuh"

static double from_bits(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t to_bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

int main(int argc, char **argv)
{
    const long long count = argc > 1 ? atoll(argv[1]) : 2000000;
    std::mt19937_64 g(4321);
    const uint64_t MANT = (1ull << 52) - 1;
    long long bad = 0, claimed = 0, special_claimed = 0;
    for (long long i = 0; i < count; i++) {
        uint64_t h1 = g(), h2 = g(), h3 = g();
        uint64_t ma = h1 & MANT, mb = h2 & MANT;
        uint32_t ea = 1 + (uint32_t)(h3 % 2046), eb = 1 + (uint32_t)((h3 >> 16) % 2046);
        switch (i % 8) {
        case 0: break;                                                  // anywhere
        case 1: ea = 1023 + (uint32_t)(h3 % 40) - 20; eb = 1023 + (uint32_t)((h3 >> 8) % 40) - 20; break;
        case 2: ea = 1023 + 500 + (uint32_t)(h3 % 30); eb = 1023 + 500 - 12 + (uint32_t)((h3 >> 8) % 30); break;  // near overflow
        case 3: ea = 1023 - 511 + (uint32_t)(h3 % 10); eb = 1023 - 511 + (uint32_t)((h3 >> 8) % 10); break;  // near underflow
        case 4: ma &= ~((1ull << (h3 % 52)) - 1); mb &= ~((1ull << ((h3 >> 8) % 52)) - 1); break;  // trailing zeros
        case 5: ma |= MANT >> (h3 % 20); mb |= MANT >> ((h3 >> 8) % 20); break;                     // runs of ones
        case 6: ma = (h3 & 1) ? 0 : ma; mb = (h3 & 2) ? 0 : mb; break;                            // powers of two
        case 7: {                                                       // specials
            const uint64_t sp[] = {0ull, 1ull, MANT, 0x7ff0000000000000ull, 0x7ff8000000000001ull,
                                   0x0010000000000000ull, 0x7fefffffffffffffull, 0x3ff0000000000000ull};
            const double a = from_bits(sp[h3 % 8] | ((h3 >> 40) & 1 ? 1ull << 63 : 0));
            const double b = from_bits((to_bits(1.0 + (double)(h1 % 1000) / 7.0)) | ((h3 >> 41) & 1 ? 1ull << 63 : 0));
            bool ok;
            const double q = nsg::mul_rn_int(a, b, ok);
            const double w = a * b;
            if (ok) { claimed++; if (to_bits(q) != to_bits(w)) { if (bad < 5) printf("BAD %a * %a: %a vs %a\n", a, b, q, w); bad++; } }
            const uint32_t e = (uint32_t)(to_bits(a) >> 52) & 0x7ff;
            if (ok && (e == 0 || e == 0x7ff)) special_claimed++;
            continue;
        }
        }
        const uint64_t sa = (h1 >> 63) << 63, sb = (h2 >> 63) << 63;
        const double a = from_bits(sa | ((uint64_t)ea << 52) | ma);
        const double b = from_bits(sb | ((uint64_t)eb << 52) | mb);
        bool ok;
        const double q = nsg::mul_rn_int(a, b, ok);
        const double w = a * b;
        if (ok) {
            claimed++;
            if (to_bits(q) != to_bits(w)) {
                if (bad < 5) printf("BAD %a * %a: %a vs %a\n", a, b, q, w);
                bad++;
            }
        } else {
            // declining is only allowed outside the normal range
            const uint64_t wb = to_bits(w);
            const uint32_t we = (uint32_t)(wb >> 52) & 0x7ff;
            // a normal product may be declined only when its unrounded exponent fell
            // below the normal range and rounding lifted it to the smallest binade
            if (we > 1 && we != 0x7ff) {
                if (bad < 5) printf("DECLINED %a * %a = %a\n", a, b, w);
                bad++;
            }
        }
    }
    printf("mismatches %lld, claimed %lld of %lld, specials claimed %lld\n", bad, claimed, count, special_claimed);
    return (bad == 0 && special_claimed == 0) ? 0 : 1;
}
