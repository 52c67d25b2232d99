// Host check of the integer-pipe tap products (wabbit_gb300/csrc/exact.cuh)
// against the host's IEEE double multiply: every product not flagged bad must
// be bit-identical, and bad may only be flagged for subnormal, infinite or NaN
// inputs or results at the ends of the normal range.
#include "exact.cuh"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

static uint64_t rng = 0x9e3779b97f4a7c15ULL;
static uint64_t next() {   // SplitMix64
    uint64_t z = (rng += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static double from_bits(uint64_t b) {
    double x;
    std::memcpy(&x, &b, 8);
    return x;
}
static uint64_t bits(double x) {
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
}

int main(int argc, char **argv) {
    const long per = argc > 1 ? std::atol(argv[1]) : 200000;
    const double taps[] = {1.0 / 16, 9.0 / 16, 1.0 / 512, 9.0 / 256, 1.0 / 32, 63.0 / 512, 9.0 / 32, 87.0 / 128,
                           3.0 / 256, 25.0 / 256, 75.0 / 128, 49.0 / 2048, 245.0 / 2048, 5.0 / 2048, 1.0, 0.5,
                           3.0, 127.0 / 64, 0.1, 1225.0 / 2048, 0.75, 5.0 / 8};
    long checked = 0, fail = 0, flagged = 0, kinds[4] = {0, 0, 0, 0};
    for (double t0 : taps)
        for (int sgn_tap = 0; sgn_tap < 2; sgn_tap++) {
            const double c = sgn_tap ? -t0 : t0;
            int kind, sh, mul;
            wg::classify_tap(c, kind, sh, mul);
            kinds[kind]++;
            if (kind == 0) continue;
            if (kind == 2 && c != 1.0) { fail++; continue; }
            const long long sg = c < 0 ? (long long)0x8000000000000000ULL : 0LL;
            for (long i = 0; i < per; i++) {
                double x;
                const int mode = (int)(i % 4);
                if (mode == 0) x = from_bits(next());                     // any pattern
                else if (mode == 1) x = std::ldexp((double)(next() >> 11) / 9007199254740992.0 + 0.5,
                                                   (int)(next() % 80) - 40) * ((next() & 1) ? -1 : 1);
                else if (mode == 2) x = from_bits((next() & 0x800fffffffffffffULL) | ((uint64_t)(next() % 2047) << 52));
                else {
                    // significands with long runs of low zero or one bits (ties, carries)
                    uint64_t f = next() & 0xfffffffffffffULL;
                    f = (next() & 1) ? (f & ~0xfffULL) : (f | 0xfffULL);
                    x = from_bits(f | ((uint64_t)(1 + next() % 2045) << 52) | ((next() & 1) << 63));
                }
                bool bad = false;
                const double r = wg::tap_mul(x, c, kind, sh, mul, sg, bad);
                const double ref = x * c;
                checked++;
                if (bad) {
                    flagged++;
                    const bool allowed = !(std::isnormal(x) || x == 0.0) || !std::isnormal(ref) ||
                                         std::fabs(ref) >= std::ldexp(1.0, 1022);
                    if (!allowed) {
                        if (fail < 10) std::printf("unexpected bad: x=%a c=%a\n", x, c);
                        fail++;
                    }
                    continue;
                }
                // NaN payloads are not part of the contract (the device returns
                // a canonical NaN)
                if (std::isnan(ref) ? !std::isnan(r) : bits(r) != bits(ref)) {
                    if (fail < 10) std::printf("mismatch: x=%a c=%a got %a want %a\n", x, c, r, ref);
                    fail++;
                }
            }
        }
    std::printf("checked %ld flagged %ld failures %ld kinds %ld %ld %ld %ld\n", checked, flagged, fail, kinds[0],
                kinds[1], kinds[2], kinds[3]);
    return fail ? 1 : 0;
}
