// Host check of the division routines of nsg_div.cuh against the CPU's IEEE
// division: every operand pair of normal numbers whose routine claims a result must
// give the same bits.  The reciprocal estimate of div_rn_lat is perturbed by
// k ulps (k from the command line) to exercise the error bounds of its digits.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

static float g_rcp_scale = 1.0f;
static inline float perturbed_rcp(int32_t x) { return (1.0f / (float)x) * g_rcp_scale; }
#define NSG_DIV_HOST_RCP perturbed_rcp
#include "nsg_div.cuh"

static double from_bits(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t to_bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

int main(int argc, char **argv)
{
    const int k = argc > 1 ? atoi(argv[1]) : 0;
    const long long count = argc > 2 ? atoll(argv[2]) : 2000000;
    g_rcp_scale = 1.0f + (float)k * 0x1p-23f;
    std::mt19937_64 g(1234 + k);
    const uint64_t MANT = (1ull << 52) - 1;
    long long bad = 0, claimed = 0, fast = 0;
    for (long long i = 0; i < count; i++) {
        uint64_t h1 = g(), h2 = g(), h3 = g();
        uint64_t ma = h1 & MANT, mb = h2 & MANT;
        switch (i % 6) {
        case 1: ma |= MANT ^ 0xff; break;                 // all-ones dividend
        case 2: mb &= ~((1ull << 40) - 1); break;         // few-bit divisor
        case 3: mb = ma; break;                           // equal mantissas
        case 4: mb = 0; break;                            // power-of-two divisor
        default: break;
        }
        const uint64_t ea = 1023 - 300 + (h3 % 600), eb = 1023 - 300 + ((h3 >> 20) % 600);
        double a = from_bits(((h3 >> 63) << 63) | (ea << 52) | ma), b = from_bits((eb << 52) | mb);
        if (i % 6 == 5) a = b * (double)((h1 >> 40) + 1);   // exact and near-exact quotients
        if (i % 97 == 0) a = (h1 & 1) ? -0.0 : 0.0;          // signed zero dividends
        const double ref = a / b;
        bool ok;
        const double q = nsg::div_rn_lat(a, b, ok);
        if (ok) {
            claimed++;
            if (to_bits(q) != to_bits(ref)) {
                if (bad < 5) printf("div_rn_lat: %a / %a = %a, IEEE %a\n", a, b, q, ref);
                bad++;
            }
        }
        double qf;
        if (nsg::div_rn_fast(a, b, &qf)) {
            fast++;
            if (to_bits(qf) != to_bits(ref)) {
                if (bad < 5) printf("div_rn_fast: %a / %a = %a, IEEE %a\n", a, b, qf, ref);
                bad++;
            }
        }
    }
    printf("perturbation %d ulp: %lld pairs, lat claimed %lld, fast claimed %lld, mismatches %lld\n", k, count,
           claimed, fast, bad);
    return bad == 0 ? 0 : 1;
}
