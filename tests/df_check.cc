// CPU check of the double-float gradients of poorly shaped elements
// (grad_df.cuh) against the FP64 gradients rounded to FP32: elements of a
// jittered unit-spaced grid at coordinates up to 1 (spacing h), flattened until
// their quality |6V| / (|a||b||c|) falls to 1e-1 .. 1e-7, coordinates split into
// FP32 hi + lo parts as the library splits them.  grad_df hands elements below
// quality 1e-4 back to the FP64 formula: a refusal above 2e-4 counts as a
// failure, and so does an error above the bound for an element it accepts.
// The error of each component is measured against the FP64 value, relative to
// the element's largest gradient component (near-zero components come from
// cancellation inside one cross product and carry absolute, not relative,
// errors in any precision): FP32 rounding alone gives up to 2^-24.
// Usage: df_check <elements> <seed>; prints
// "<checked> <max error / 2^-24> <failures> <refused below 1e-4>".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "grad_df.cuh"

static unsigned long long state;
static double urand() {
    unsigned long long z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// FP64 gradients: the reference's formula (edge vectors, cross products, 1/vol)
static bool grad64(const double x[4][3], double g[12]) {
    double a[3], b[3], c[3];
    for (int k = 0; k < 3; k++) {
        a[k] = x[0][k] - x[3][k];
        b[k] = x[2][k] - x[3][k];
        c[k] = x[1][k] - x[3][k];
    }
    double G[12];
    G[0] = b[1] * c[2] - c[1] * b[2]; G[1] = b[2] * c[0] - c[2] * b[0]; G[2] = b[0] * c[1] - c[0] * b[1];
    G[3] = a[1] * b[2] - b[1] * a[2]; G[4] = a[2] * b[0] - b[2] * a[0]; G[5] = a[0] * b[1] - b[0] * a[1];
    G[6] = c[1] * a[2] - a[1] * c[2]; G[7] = c[2] * a[0] - a[2] * c[0]; G[8] = c[0] * a[1] - a[0] * c[1];
    for (int k = 0; k < 3; k++) G[9 + k] = -((G[k] + G[3 + k]) + G[6 + k]);
    const double vol = (a[0] * G[0] + a[1] * G[1]) + a[2] * G[2];
    if (vol == 0.0) return false;
    const double r = 1.0 / vol;
    for (int i = 0; i < 12; i++) g[i] = G[i] * r;
    return true;
}

int main(int argc, char **argv) {
    const long long n = argc > 1 ? std::atoll(argv[1]) : 100000;
    state = argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 1;
    long long checked = 0, over = 0, refused = 0;
    double worst = 0.0;
    for (long long it = 0; it < n; it++) {
        const double h = 0.002 + 0.05 * urand();
        double x[4][3];
        const double o[3] = {urand(), urand(), urand()};
        const double ref[4][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {1, 1, 1}};
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 3; k++) x[j][k] = o[k] + h * (ref[j][k] + 0.3 * (urand() - 0.5));
        // flatten: move node 3 towards the plane of nodes 0, 1, 2
        const double t = std::pow(10.0, -7.0 * urand());
        double ctr[3];
        for (int k = 0; k < 3; k++) ctr[k] = (x[0][k] + x[1][k] + x[2][k]) / 3.0;
        for (int k = 0; k < 3; k++) x[3][k] = ctr[k] + t * (x[3][k] - ctr[k]);
        float hi[4][3], lo[4][3];
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 3; k++) {
                hi[j][k] = (float)x[j][k];
                lo[j][k] = (float)(x[j][k] - (double)hi[j][k]);
            }
        double g64[12];
        float g[12];
        if (!grad64(x, g64)) continue;
        double a[3], b[3], c[3];
        for (int k = 0; k < 3; k++) {
            a[k] = x[0][k] - x[3][k];
            b[k] = x[2][k] - x[3][k];
            c[k] = x[1][k] - x[3][k];
        }
        const double vol = a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
                           a[2] * (b[0] * c[1] - b[1] * c[0]);
        const double q = std::fabs(vol) / std::sqrt((a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) *
                                                    (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) *
                                                    (c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
        if (!mfem::grad_df(hi, lo, g)) {
            if (q > 2e-4) {
                if (over < 5) std::printf("# elem %lld refused at quality %.3g\n", it, q);
                over++;
            } else {
                refused++;
            }
            continue;
        }
        checked++;
        double gmax = 0.0;
        for (int i = 0; i < 12; i++) gmax = std::fmax(gmax, std::fabs(g64[i]));
        for (int i = 0; i < 12; i++) {
            const double e = std::fabs((double)g[i] - g64[i]) / gmax * 16777216.0;   // in units of 2^-24
            if (e > worst) worst = e;
            if (e > 1.5) {
                if (over < 5) std::printf("# elem %lld comp %d: %.9g vs %.17g (t %.3g)\n", it, i, g[i], g64[i], t);
                over++;
            }
        }
    }
    std::printf("%lld %.3f %lld %lld\n", checked, worst, over, refused);
    return over ? 1 : 0;
}
