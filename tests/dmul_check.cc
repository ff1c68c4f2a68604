// CPU check of the integer-pipe double multiplication and hi/lo split (the
// header's portable path) against the host's IEEE arithmetic: random bit
// patterns, operands near 1.0, short significands (ties), exhaustive
// small-integer products, and splits with ties in the dropped bits.
// Usage: dmul_check <pairs> <seed>; prints "<fast> <mismatches>".
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "dmul_int.cuh"

static uint64_t state;
static uint64_t next() {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double as_double(uint64_t u) { double x; std::memcpy(&x, &u, 8); return x; }
static uint64_t as_bits(double x) { uint64_t u; std::memcpy(&u, &x, 8); return u; }

int main(int argc, char **argv) {
    const long long n = argc > 1 ? std::atoll(argv[1]) : 1000000;
    state = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    unsigned long long fast = 0, bad = 0;
    auto check = [&](uint64_t A, uint64_t B) {
        uint64_t r;
        if (!mfem::dmul_bits(A, B, &r)) return;
        fast++;
        volatile double a = as_double(A), b = as_double(B);
        const double ref = a * b;
        if (r != as_bits(ref)) {
            if (bad < 5) std::printf("# %016llx * %016llx: %016llx != %016llx\n",
                                     (unsigned long long)A, (unsigned long long)B,
                                     (unsigned long long)r, (unsigned long long)as_bits(ref));
            bad++;
        }
    };
    for (long long i = 0; i < n; i++) {
        uint64_t A = next(), B = next();
        switch (i % 3) {
        case 1:
            A = (A & 0x800fffffffffffffull) | ((uint64_t)(973 + (A >> 20) % 100) << 52);
            B = (B & 0x800fffffffffffffull) | ((uint64_t)(973 + (B >> 20) % 100) << 52);
            break;
        case 2: {
            const int ka = (int)(A % 27), kb = (int)(B % 27);
            A = (A & (0x000fffffffffffffull << ka) & 0x800fffffffffffffull) | (1000ull << 52);
            B = (B & (0x000fffffffffffffull << kb) & 0x800fffffffffffffull) | (1030ull << 52);
            break;
        }
        default:
            break;
        }
        check(A, B);
    }
    for (uint64_t x = 1; x < 2048; x++)
        for (uint64_t y = 1; y < 2048; y++)
            check(as_bits((double)x * 1.5), as_bits((double)(9007199254740992ull - y)));
    // hi/lo split of doubles: fl32(x) and fl32(x - fl32(x)), random patterns
    // with exponents around 1.0 and ties of the 29 dropped bits
    for (long long i = 0; i < n; i++) {
        uint64_t X = next();
        X = (X & 0x800fffffffffffffull) | ((uint64_t)(963 + (X >> 40) % 161) << 52);
        if (i % 4 == 1) X = (X & ~0x1fffffffull) | 0x10000000ull;        // exact tie
        if (i % 4 == 2) X &= ~0x1fffffffull;                             // exact in FP32
        uint32_t h, l;
        if (!mfem::split_f32_bits(X, &h, &l)) continue;
        fast++;
        volatile double x = as_double(X);
        const float rh = (float)x;
        volatile double rest = x - (double)rh;
        const float rl = (float)rest;
        uint32_t bh, bl;
        std::memcpy(&bh, &rh, 4);
        std::memcpy(&bl, &rl, 4);
        if (h != bh || l != bl) {
            if (bad < 5) std::printf("# split %016llx: %08x %08x != %08x %08x\n",
                                     (unsigned long long)X, h, l, bh, bl);
            bad++;
        }
    }
    std::printf("%llu %llu\n", fast, bad);
    return bad != 0;
}
