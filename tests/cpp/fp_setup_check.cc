// Host build of the forward projector's per-ray set-up (fp_setup.cuh),
// checked ray by ray against the reference's FP64 inclusion rule.
// Input (binary, stdin): int32 n, int32 nrays, then nrays x (begin, step) FP64.
// Output: "rays fixed split fallback mismatch_fma mismatch_acc bad_index".
// With the argument "conv": checks dbl2flt against the compiler's conversion on
// random doubles and prints the number of mismatches.  With "col": reads the
// same input and checks col_range, for every ray taken as a column ray and
// several band heights, against the brute-force sample set, plus random
// lines with tiny, zero and negative steps; prints the number of mismatches.
// With "acc": checks acc_advance against the plain FP64 loop on random
// starts, steps and checkpoints; prints "cases mismatches".
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <random>
#include <vector>

#include "../../ct_recon_extensions_gb300/csrc/fp_setup.cuh"

static int conv_check()
{
    std::mt19937_64 rng(7);
    long long bad = 0;
    for (int i = 0; i < 2000000; ++i) {
        unsigned long long b = rng();
        const int e = static_cast<int>((b >> 52) & 0x7FF);
        if (e == 0x7FF) continue;                     // inf / nan
        double v;
        std::memcpy(&v, &b, 8);
        if (std::fabs(v) < 1.2e-38 || std::fabs(v) > 3.0e38) continue;  // float normal range
        const float a = ctr::dbl2flt(v), r = static_cast<float>(v);
        if (std::memcmp(&a, &r, 4) != 0) ++bad;
    }
    // values near 1 and exact halfway cases
    for (int i = 0; i < 1000000; ++i) {
        const double v = std::ldexp(static_cast<double>(rng() >> 11), -53) * (i & 1 ? 7.0 : -0.3);
        if (std::fabs(v) < 1.2e-38) continue;
        const float a = ctr::dbl2flt(v), r = static_cast<float>(v);
        if (std::memcmp(&a, &r, 4) != 0) ++bad;
    }
    std::printf("%lld\n", bad);
    return 0;
}


static long long col_one(long long X0, long long S, int n, int k0, int k1)
{
    long long bad = 0;
    static const int bands[] = {1, 2, 7, 15, 32};
    for (int band : bands) {
        std::vector<int> seen(n, 0);
        for (int b0 = 0; b0 < n; b0 += band) {
            const int b1 = std::min(b0 + band, n) - 1;
            int ia, ib;
            ctr::col_range(X0, S, b0, b1, k0, k1, &ia, &ib);
            const long long B0 = static_cast<long long>(b0) << 32, B1 = static_cast<long long>(b1 + 1) << 32;
            int ta = k1 + 1, tb = k1;  // brute force (a contiguous set)
            for (int ix = k0; ix <= k1; ++ix) {
                const long long y = X0 + static_cast<long long>(ix) * S;
                if (y >= B0 && y < B1) {
                    if (ta > k1) ta = ix;
                    tb = ix;
                }
            }
            const bool empty_t = ta > tb, empty_c = ia > ib;
            if (empty_t != empty_c || (!empty_t && (ia != ta || ib != tb))) ++bad;
            if (!empty_c)
                for (int ix = ia; ix <= ib && ix >= 0 && ix < n; ++ix) ++seen[ix];
        }
        for (int ix = 0; ix < n; ++ix) {
            const long long y = X0 + static_cast<long long>(ix) * S;
            const bool valid = ix >= k0 && ix <= k1 && y >= 0 && y < (static_cast<long long>(n) << 32);
            if (seen[ix] != (valid ? 1 : 0)) ++bad;
        }
    }
    return bad;
}

static int col_check()
{
    int n = 0, nr = 0;
    if (std::fread(&n, 4, 1, stdin) != 1 || std::fread(&nr, 4, 1, stdin) != 1) return 2;
    std::vector<double> t(2 * static_cast<size_t>(nr));
    if (std::fread(t.data(), 8, t.size(), stdin) != t.size()) return 2;
    long long bad = 0;
    for (int r = 0; r < nr; r += 7) {
        long long X0, S;
        int k0, k1, amb[4], namb;
        if (!ctr::ray_fixed(t[2 * r], t[2 * r + 1], n, &X0, &S, &k0, &k1) &&
            !ctr::ray_split(t[2 * r], t[2 * r + 1], n, &X0, &S, &k0, &k1, amb, &namb))
            ctr::ray_fp64(t[2 * r], t[2 * r + 1], n, &X0, &S, &k0, &k1);
        if (k0 <= k1) bad += col_one(X0, S, n, k0, k1);
    }
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const double steps[] = {0.0, 1e-9, -1e-9, 3e-6, -2e-4, 0.03, -0.7, 1.0, -1.0};
    for (int i = 0; i < 3000; ++i) {
        const double step = i < 900 ? steps[i % 9] : (U(rng) * 2.0 - 1.0);
        const double y0 = U(rng) * (n - 1);
        const long long X0 = std::llrint(y0 * ctr::kFix32), S = std::llrint(step * ctr::kFix32);
        // the samples with Y inside [0, n-1]
        int k0 = n, k1 = -1;
        for (int ix = 0; ix < n; ++ix) {
            const long long y = X0 + static_cast<long long>(ix) * S;
            if (y >= 0 && y <= (static_cast<long long>(n - 1) << 32)) {
                if (k0 == n) k0 = ix;
                k1 = ix;
            }
        }
        if (k0 <= k1) bad += col_one(X0, S, n, k0, k1);
    }
    std::printf("%lld\n", bad);
    return 0;
}

static int acc_check()
{
    std::mt19937_64 rng(5);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    long long bad = 0, cases = 0;
    for (int i = 0; i < 200000; ++i) {
        double begin, step;
        const int kind = i % 6;
        if (kind == 0) {        // prep-like: begin in [-600, 1100], |step| <= 1
            begin = U(rng) * 1700.0 - 600.0;
            step = U(rng) * 2.0 - 1.0;
        } else if (kind == 1) { // through zero with small steps
            begin = (U(rng) - 0.5) * 4.0;
            step = (U(rng) - 0.5) * 0.01;
        } else if (kind == 2) { // exact grid values (ties at pixel centres)
            begin = std::floor(U(rng) * 64.0) - 20.0;
            step = (i & 8) ? 1.0 : -1.0;
            if (i & 16) step = std::nextafter(step, 0.0);
        } else if (kind == 3) { // tiny steps
            begin = U(rng) * 512.0;
            step = (U(rng) - 0.5) * 1e-12;
        } else if (kind == 4) { // steps with a half-ulp remainder pattern
            begin = std::ldexp(1.0, static_cast<int>(U(rng) * 10)) + std::floor(U(rng) * 100);
            step = std::ldexp(1.0, -static_cast<int>(U(rng) * 50)) * 3.0;
        } else {                // random scale
            begin = std::ldexp(U(rng) - 0.5, static_cast<int>(U(rng) * 24) - 12);
            step = std::ldexp(U(rng) - 0.5, static_cast<int>(U(rng) * 24) - 14);
        }
        const int K = 1 + static_cast<int>(U(rng) * 2048);
        // checkpoints: a few targets along the way, as the kernel asks for them
        ctr::AccWalk w{begin, 0};
        double x = begin;
        int k = 0;
        for (int c = 0; c < 4; ++c) {
            const int target = std::min(K, w.k + 1 + static_cast<int>(U(rng) * K / 2));
            ctr::acc_advance(&w, step, target);
            while (k < target) {
                x += step;
                ++k;
            }
            ++cases;
            if (std::memcmp(&x, &w.x, 8) != 0 || w.k != k) ++bad;
        }
    }
    std::printf("%lld %lld\n", cases, bad);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc > 1 && std::strcmp(argv[1], "acc") == 0) return acc_check();
    if (argc > 1 && std::strcmp(argv[1], "conv") == 0) return conv_check();
    if (argc > 1 && std::strcmp(argv[1], "col") == 0) return col_check();
    int n = 0, nr = 0;
    if (std::fread(&n, 4, 1, stdin) != 1 || std::fread(&nr, 4, 1, stdin) != 1) return 2;
    std::vector<double> t(2 * static_cast<size_t>(nr));
    if (std::fread(t.data(), 8, t.size(), stdin) != t.size()) return 2;
    const long long L = static_cast<long long>(n - 1) << 32;
    long long fixed = 0, split = 0, fallback = 0, mis_fma = 0, mis_acc = 0, bad = 0;
    for (int r = 0; r < nr; ++r) {
        const double begin = t[2 * r], step = t[2 * r + 1];
        long long X0, S;
        int k0, k1, amb[4], namb = 0;
        bool is_split = false;
        if (ctr::ray_fixed(begin, step, n, &X0, &S, &k0, &k1)) {
            ++fixed;
        } else if (ctr::ray_split(begin, step, n, &X0, &S, &k0, &k1, amb, &namb)) {
            ++split;
            is_split = true;
        } else {
            ++fallback;
            ctr::ray_fp64(begin, step, n, &X0, &S, &k0, &k1);
        }
        double xacc = begin;  // the reference accumulates x += step
        for (int k = 0; k < n; ++k) {
            const double xf = std::fma(static_cast<double>(k), step, begin);
            const bool vf = xf >= 0.0 && xf <= n - 1;
            const bool va = xacc >= 0.0 && xacc <= n - 1;
            bool v = k >= k0 && k <= k1;
            bool streamed = v;
            if (is_split)
                for (int a = 0; a < namb; ++a)
                    if (amb[a] == k && ctr::acc_inside(begin, step, n, k)) v = true;
            mis_fma += v != vf;
            mis_acc += v != va;
            if (streamed) {
                const long long X = X0 + static_cast<long long>(k) * S;
                const long long hi = X >> 32;
                // reads p[hi] and p[hi + 1]: hi in [0, n-1]; hi == n-1 only a hair above L
                if (X < 0 || hi > n - 1 || (hi == n - 1 && X - L > n)) ++bad;
                const double xr = static_cast<double>(X) / ctr::kFix32;
                if (std::fabs(xr - xf) > 1e-6) ++bad;
            }
            xacc += step;
        }
    }
    std::printf("%d %lld %lld %lld %lld %lld %lld\n", nr, fixed, split, fallback, mis_fma, mis_acc, bad);
    return 0;
}
