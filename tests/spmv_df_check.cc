// CPU check of the double-float accumulation of the FP32-valued operator
// (spmv_df.cuh) in the order k_spmv32 uses: four lanes per block row, blocks
// taken in chunks of 8 (lane l the blocks l and l + 4 of each chunk), each
// lane's products summed in block, row, column order and its pair renormalized
// after each chunk, the lanes merged by the
// xor butterfly (offsets 2, then 1), lane d's pair giving component d.  x is
// scaled by the power of two that brings max |x| below 1 and split into FP32
// hi + lo parts by rounding; the result (s + t) 2^kx is compared with the exact
// sum of a x (FP64 products split exactly by FMA, summed as a Shewchuk
// expansion), the error measured relative to the row's sum of |a x| in units
// of 2^-48.  Rows: random FP32 blocks whose rows sum to zero (as the assembled
// operators' do on constant fields) with x either random or a constant plus a
// small perturbation (heavy cancellation), x spanning up to 2^-30 of max |x|.
// Usage: spmv_df_check <rows> <seed> <dim>; prints
// "<components checked> <max error / 2^-48> <mean error / 2^-48>".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "spmv_df.cuh"

static unsigned long long state;
static double urand() {
    unsigned long long z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// Shewchuk's exact expansion of a sum of doubles, then summed smallest first
struct Expansion {
    std::vector<double> p;
    void add(double x) {
        size_t i = 0;
        for (double y : p) {
            if (std::fabs(x) < std::fabs(y)) std::swap(x, y);
            const double hi = x + y;
            const double lo = y - (hi - x);
            if (lo != 0.0) p[i++] = lo;
            x = hi;
        }
        p.resize(i);
        p.push_back(x);
    }
    double value() const {
        double s = 0.0;
        for (double v : p) s += v;
        return s;
    }
};

int main(int argc, char **argv) {
    const long long nRows = argc > 1 ? std::atoll(argv[1]) : 10000;
    state = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    const int D = argc > 3 ? std::atoi(argv[3]) : 3;
    const int B = D * D, kLanes = 4, kChunk = 8;
    long long checked = 0;
    double worst = 0.0, total = 0.0;
    for (long long r = 0; r < nRows; r++) {
        const int nb = 1 + (int)(urand() * 40);
        std::vector<float> a((size_t)nb * B);
        for (auto &v : a) v = (float)((2.0 * urand() - 1.0) * std::ldexp(1.0, (int)(urand() * 20) - 10));
        // rows of the first block make every row sum to zero
        for (int i = 0; i < D; i++)
            for (int j = 0; j < D; j++) {
                double s = 0.0;
                for (int k = 1; k < nb; k++) s += a[(size_t)k * B + D * i + j];
                a[D * i + j] = (float)(-s);
            }
        const bool smooth = urand() < 0.5;
        const double c = 2.0 * urand() - 1.0;
        std::vector<double> x((size_t)nb * D);
        for (auto &v : x) {
            const double u = 2.0 * urand() - 1.0;
            v = smooth ? c + 1e-6 * u : u * std::ldexp(1.0, -(int)(urand() * 30));
        }
        double xmax = 0.0;
        for (double v : x) xmax = std::fmax(xmax, std::fabs(v));
        int kx = 0;
        if (xmax > 0.0) std::frexp(xmax, &kx);   // 2^(kx-1) <= xmax < 2^kx
        std::vector<float> xh(x.size()), xl(x.size());
        for (size_t k = 0; k < x.size(); k++) {
            const double v = std::ldexp(x[k], -kx);
            xh[k] = (float)v;
            xl[k] = (float)(v - (double)xh[k]);
        }
        float s[4][3] = {}, t[4][3] = {};
        for (int lane = 0; lane < kLanes; lane++)
            for (int k0 = 0; k0 < nb; k0 += kChunk) {
                for (int j = 0; j < kChunk / kLanes; j++) {
                    const int k = k0 + lane + kLanes * j;
                    if (k >= nb) continue;
                    for (int i = 0; i < D; i++)
                        for (int jj = 0; jj < D; jj++)
                            mfem::spdf::accumulate(s[lane][i], t[lane][i], a[(size_t)k * B + D * i + jj],
                                                   xh[(size_t)k * D + jj], xl[(size_t)k * D + jj]);
                }
                for (int i = 0; i < D; i++) mfem::spdf::renormalize(s[lane][i], t[lane][i]);
            }
        for (int off = kLanes / 2; off >= 1; off >>= 1) {
            float ns[4][3], nt[4][3];
            for (int lane = 0; lane < kLanes; lane++)
                for (int d = 0; d < D; d++) {
                    ns[lane][d] = s[lane][d];
                    nt[lane][d] = t[lane][d];
                    mfem::spdf::merge(ns[lane][d], nt[lane][d], s[lane ^ off][d], t[lane ^ off][d]);
                }
            for (int lane = 0; lane < kLanes; lane++)
                for (int d = 0; d < D; d++) {
                    s[lane][d] = ns[lane][d];
                    t[lane][d] = nt[lane][d];
                }
        }
        for (int d = 0; d < D; d++) {
            Expansion e;
            double mag = 0.0;
            for (int k = 0; k < nb; k++)
                for (int jj = 0; jj < D; jj++) {
                    const double av = (double)a[(size_t)k * B + D * d + jj], xv = x[(size_t)k * D + jj];
                    const double p = av * xv;
                    e.add(p);
                    e.add(std::fma(av, xv, -p));
                    mag += std::fabs(p);
                }
            if (mag == 0.0) continue;
            const double y = std::ldexp((double)s[d][d] + (double)t[d][d], kx);
            const double err = std::fabs(y - e.value()) / mag * std::ldexp(1.0, 48);
            worst = std::fmax(worst, err);
            total += err;
            checked++;
        }
    }
    std::printf("%lld %.4f %.4f\n", checked, worst, checked ? total / checked : 0.0);
    return 0;
}
