// Host check of pd_gpu1_gb300/csrc/exact_sub.h against the hardware double
// subtraction: random operand pairs of the same sign within a factor of two,
// both in one binade and straddling a power of two, plus the refused cases.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "exact_sub.h"

static uint64_t bits(double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    return u;
}
int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.5, 2.0);
    long bad = 0, used = 0, refused = 0;
    for (long i = 0; i < 2000000; i++) {
        const double scale = std::ldexp(1.0, (int)(rng() % 60) - 40);
        double a = U(rng) * scale;
        double b = a * U(rng) * 0.999 + (i % 7 == 0 ? std::ldexp(1.0, (int)(rng() % 20) - 60) : 0.0);
        if (i % 5 == 0) {  // straddle a power of two
            a = std::ldexp(1.0 + 1e-9 * (double)(rng() % 1000), (int)(rng() % 40) - 30);
            b = std::ldexp(1.0 - 1e-9 * (double)(rng() % 1000), std::ilogb(a));
        }
        if (i & 1) {
            a = -a;
            b = -b;
        }
        uint64_t r;
        if (!pdg::sub_exact(bits(a), bits(b), r)) {
            refused++;
            continue;
        }
        used++;
        const double want = a - b;
        // exact by Sterbenz when b/2 <= a <= 2b; elsewhere the helper must refuse or agree
        if (r != bits(want) && !(want == 0.0 && r == 0)) {
            if (std::fabs(a) <= 2 * std::fabs(b) && std::fabs(b) <= 2 * std::fabs(a)) bad++;
        }
        int64_t diff;
        int e;
        pdg::sub_exact_scaled(bits(a), bits(b), diff, e);
        if (std::ldexp((double)diff, e - 1075) != want && std::llabs(diff) < (1ll << 53)) bad++;
    }
    uint64_t r;
    const bool refuse_sign = !pdg::sub_exact(bits(1.0), bits(-1.0), r);
    const bool refuse_zero = !pdg::sub_exact(bits(0.0), bits(1.0), r);
    const bool refuse_far = !pdg::sub_exact(bits(8.0), bits(1.0), r);
    std::printf("used %ld refused %ld bad %ld refuse_sign %d refuse_zero %d refuse_far %d\n", used, refused, bad,
                refuse_sign, refuse_zero, refuse_far);
    return (bad == 0 && refuse_sign && refuse_zero && refuse_far && used > 1000000) ? 0 : 1;
}
