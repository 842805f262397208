// Per-ray set-up of the FP32 ray-driven forward projector: the ray's sample
// range and its 32.32 fixed-point line, from the caller's FP64 table entry
// (begin, step) of the reference's prep (src/fp_par_2d.cc:180-199).  The _n
// forms take the number of samples n and the extent ext of the axis (samples
// valid iff 0 <= x(k) <= ext-1) separately: the ray-casting projector walks one
// axis of a 2-D ray with n != ext; the plain forms are n == ext.
//
// A sample k of the ray sits at x(k) = begin + k*step (pixel units along the
// marched row); it is used iff 0 <= x(k) <= n-1 (src/fp_par_2d.cc:237,259).
// The common path decides this in integer arithmetic on
// X(k) = fix(begin) + k*fix(step), fix(v) = round(v * 2^32), which is within
// 0.5 + 0.5k units of x(k) * 2^32.  Where an end sample (or the first sample
// outside) lies within tie_units(n) of 0 or n-1, or the magnitudes are out of
// the exact range, the caller takes ray_fp64 instead, which applies the
// reference's own accumulated FP64 rule; so the decisions are the reference's
// in every case.
//
// Plain C++ with a __host__ __device__ qualifier, so a host build of the same
// code can be checked against the FP64 rule on the CPU.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define CTR_HD __host__ __device__ __forceinline__
#else
#define CTR_HD inline
#endif

namespace ctr {

constexpr double kFix32 = 4294967296.0;  // 2^32

// Bit pattern of a double (host and device).
CTR_HD unsigned long long double_bits(double v)
{
#if defined(__CUDA_ARCH__)
    return static_cast<unsigned long long>(__double_as_longlong(v));
#else
    unsigned long long b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}

// float(v) rounded to nearest even, from the bits with integer operations (the
// FP64 unit is slow); |v| below 2^-126 gives a signed zero, above the float
// range an infinity.
CTR_HD float dbl2flt(double v)
{
    const unsigned long long b = double_bits(v);
    const unsigned sign = static_cast<unsigned>(b >> 63) << 31;
    const int e = static_cast<int>((b >> 52) & 0x7FF) - 1023 + 127;
    unsigned bits;
    if (e <= 0) {
        bits = sign;
    } else if (e >= 255) {
        bits = sign | 0x7F800000u;
    } else {
        const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
        unsigned r = (static_cast<unsigned>(e) << 23) | static_cast<unsigned>(m >> 29);
        const unsigned long long rem = m & 0x1FFFFFFFull, half = 0x10000000ull;
        if (rem > half || (rem == half && (r & 1u))) ++r;  // a carry into the exponent is right
        bits = sign | (r >= 0x7F800000u ? 0x7F800000u : r);
    }
#if defined(__CUDA_ARCH__)
    return __uint_as_float(bits);
#else
    float f;
    std::memcpy(&f, &bits, sizeof f);
    return f;
#endif
}

// round(v * 2^32) with ties to even (llrint in the default rounding mode),
// using integer operations only.  Valid for |v| < 2^20 (the caller checks).
CTR_HD long long fix32(double v)
{
    const unsigned long long bits = double_bits(v);
    const int e = static_cast<int>((bits >> 52) & 0x7FF);
    if (e == 0) return 0;  // zero or subnormal: |v * 2^32| < 2^-990
    const unsigned long long m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    // v * 2^32 = m * 2^(e - 1075 + 32) = m >> (1043 - e)
    const int sh = 1043 - e;
    unsigned long long r;
    if (sh <= 0) {
        r = m << (-sh > 10 ? 10 : -sh);  // |v| >= 2^20: excluded by the caller
    } else if (sh > 54) {
        r = 0;  // m * 2^-sh < 2^53 * 2^-55 = 0.25
    } else {
        const unsigned long long q = m >> sh;
        const unsigned long long rem = m & ((1ull << sh) - 1);
        const unsigned long long half = 1ull << (sh - 1);
        r = q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull);
    }
    const long long s = static_cast<long long>(r);
    return (bits >> 63) ? -s : s;
}

// Units of 2^-32 px within which an end sample counts as a tie.  Covers the
// fixed-point error 0.5 + 0.5k and the reference's own accumulation of x
// (< 0.2k units) with a wide margin.
CTR_HD long long tie_units(int n) { return static_cast<long long>(n) + 1024; }

// Integer sample range and fixed-point line of one ray.  Returns false when
// the ray must take the FP64 path (tie, magnitude, or an estimate that did
// not verify).  On success the valid samples are [*k0, *k1] (empty when
// *k1 < *k0) and every valid sample has tie_units(n) <= X(k) <= L - tie_units(n).
CTR_HD bool ray_fixed_n(double begin, double step, int n, int ext, long long* X0, long long* Sout,
                        int* k0o, int* k1o)
{
    // exact-range guard (also rejects NaN / Inf): |begin| < 2^20, |step| < 4
    const int eb = static_cast<int>((double_bits(begin) >> 52) & 0x7FF);
    const int es = static_cast<int>((double_bits(step) >> 52) & 0x7FF);
    if (eb >= 1043 || es >= 1025) return false;
    const long long B = fix32(begin), S = fix32(step);
    const long long L = static_cast<long long>(ext - 1) << 32;
    const long long T = tie_units(n);
    auto X = [&](int k) { return B + static_cast<long long>(k) * S; };
    auto inside = [&](int k) {
        const long long x = X(k);
        return x >= 0 && x <= L;
    };
    int k0, k1;
    if (S == 0) {
        if (inside(0)) {
            k0 = 0;
            k1 = n - 1;
        } else {
            k0 = 1;
            k1 = 0;
        }
    } else {
        // real-valued crossing points, estimated in FP32, then settled exactly
        const float fb = dbl2flt(begin), fs = dbl2flt(step);
        float ta = -fb / fs, tb = (static_cast<float>(ext - 1) - fb) / fs;
        if (ta > tb) {
            const float t = ta;
            ta = tb;
            tb = t;
        }
        const float lo = ta < -2.0f ? -2.0f : (ta > n + 2.0f ? n + 2.0f : ta);
        const float hi = tb < -2.0f ? -2.0f : (tb > n + 2.0f ? n + 2.0f : tb);
        k0 = static_cast<int>(std::ceil(lo));
        k1 = static_cast<int>(std::floor(hi));
        if (k0 < 0) k0 = 0;
        if (k1 > n - 1) k1 = n - 1;
        // settle the estimate (off by at most one here); anything else fails
        // the verification below and takes the FP64 path
        for (int it = 0; it < 3 && k0 > 0 && inside(k0 - 1); ++it) --k0;
        for (int it = 0; it < 3 && k0 <= k1 && !inside(k0); ++it) ++k0;
        for (int it = 0; it < 3 && k1 < n - 1 && inside(k1 + 1); ++it) ++k1;
        for (int it = 0; it < 3 && k1 >= k0 && !inside(k1); ++it) --k1;
    }
    if (k0 <= k1) {
        if (!inside(k0) || !inside(k1)) return false;
        if (k0 > 0 && inside(k0 - 1)) return false;
        if (k1 < n - 1 && inside(k1 + 1)) return false;
    } else {
        // empty: every sample must be on one side of [0, L]
        const long long xa = X(0), xb = X(n - 1);
        const long long mx = xa > xb ? xa : xb, mn = xa < xb ? xa : xb;
        if (!(mx < 0 || mn > L)) return false;
    }
    // ties: the samples next to either boundary
    auto near = [&](int k) {
        if (k < 0 || k > n - 1) return false;
        const long long x = X(k);
        return (x > -T && x < T) || (x > L - T && x < L + T);
    };
    if (near(0) || near(n - 1)) return false;
    if (k0 <= k1 && (near(k0 - 1) || near(k0) || near(k1) || near(k1 + 1))) return false;
    *X0 = B;
    *Sout = S;
    *k0o = k0;
    *k1o = k1;
    return true;
}

CTR_HD bool ray_fixed(double begin, double step, int n, long long* X0, long long* Sout, int* k0o,
                      int* k1o)
{
    return ray_fixed_n(begin, step, n, n, X0, Sout, k0o, k1o);
}

// For a ray that ray_fixed could not settle: the samples certainly inside
// (T <= X(k) <= L - T, decided in fixed point) as [*c0, *c1], and the
// ambiguous samples next to them (|X| < T or |X - L| < T), at most two at each
// end, in amb[0..*namb).  Their inclusion is the reference's accumulated FP64
// rule (acc_inside), which the caller evaluates separately.  Returns false when
// the ray needs ray_fp64 instead: magnitudes out of range, no certain sample,
// or a longer ambiguous run (a ray almost parallel to an image edge).
CTR_HD bool ray_split_n(double begin, double step, int n, int ext, long long* X0, long long* Sout,
                        int* c0o, int* c1o, int* amb, int* namb)
{
    const int eb = static_cast<int>((double_bits(begin) >> 52) & 0x7FF);
    const int es = static_cast<int>((double_bits(step) >> 52) & 0x7FF);
    if (eb >= 1043 || es >= 1025 || n < 4) return false;
    const long long B = fix32(begin), S = fix32(step);
    const long long L = static_cast<long long>(ext - 1) << 32;
    const long long T = tie_units(n);
    auto X = [&](int k) { return B + static_cast<long long>(k) * S; };
    auto in = [&](int k) {
        const long long x = X(k);
        return x >= T && x <= L - T;
    };
    auto amb_at = [&](int k) {
        if (k < 0 || k > n - 1) return false;
        const long long x = X(k);
        return (x > -T && x < T) || (x > L - T && x < L + T);
    };
    if (S == 0) return false;  // all samples alike: left to ray_fp64
    const float fb = dbl2flt(begin), fs = dbl2flt(step);
    const float tl = static_cast<float>(T) / 4294967296.0f;
    const float hi_x = static_cast<float>(ext - 1) - tl;
    float ta = (tl - fb) / fs, tb = (hi_x - fb) / fs;
    if (ta > tb) {
        const float t = ta;
        ta = tb;
        tb = t;
    }
    const float lo = ta < -2.0f ? -2.0f : (ta > n + 2.0f ? n + 2.0f : ta);
    const float hi = tb < -2.0f ? -2.0f : (tb > n + 2.0f ? n + 2.0f : tb);
    int c0 = static_cast<int>(std::ceil(lo)), c1 = static_cast<int>(std::floor(hi));
    if (c0 < 0) c0 = 0;
    if (c1 > n - 1) c1 = n - 1;
    for (int it = 0; it < 3 && c0 > 0 && in(c0 - 1); ++it) --c0;
    for (int it = 0; it < 3 && c0 <= c1 && !in(c0); ++it) ++c0;
    for (int it = 0; it < 3 && c1 < n - 1 && in(c1 + 1); ++it) ++c1;
    for (int it = 0; it < 3 && c1 >= c0 && !in(c1); ++it) --c1;
    if (c0 > c1 || !in(c0) || !in(c1)) return false;
    if ((c0 > 0 && in(c0 - 1)) || (c1 < n - 1 && in(c1 + 1))) return false;
    int m = 0;
    for (int k = c0 - 1; k >= c0 - 2; --k)
        if (amb_at(k)) amb[m++] = k;
    if (amb_at(c0 - 3)) return false;
    for (int k = c1 + 1; k <= c1 + 2; ++k)
        if (amb_at(k)) amb[m++] = k;
    if (amb_at(c1 + 3)) return false;
    *X0 = B;
    *Sout = S;
    *c0o = c0;
    *c1o = c1;
    *namb = m;
    return true;
}

CTR_HD bool ray_split(double begin, double step, int n, long long* X0, long long* Sout, int* c0o,
                      int* c1o, int* amb, int* namb)
{
    return ray_split_n(begin, step, n, n, X0, Sout, c0o, c1o, amb, namb);
}

// Bits -> double (host and device).
CTR_HD double bits_double(unsigned long long b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(b));
#else
    double v;
    std::memcpy(&v, &b, sizeof v);
    return v;
#endif
}

// The reference's running position: x after k steps of x += step from begin,
// each sum rounded to FP64 (src/fp_par_2d.cc:236-249), advanced from sample
// `k` to sample `target`.  Exact, with few FP64 operations: while x and its
// successor share a sign and a binade (grid u), every step adds the same
// rounded increment d = fl(x + step) - x (the sum's remainder modulo u is that
// of step, so the rounding repeats), unless the rounding is a tie (the
// remainder is u/2), so such a run is jumped over with integer arithmetic on
// the significand; the steps across binades, signs and ties are taken one by one.
struct AccWalk {
    double x;
    int k;
};

CTR_HD void acc_advance(AccWalk* w, double step, int target)
{
    double x = w->x;
    int k = w->k;
    while (k < target) {
        const double x1 = x + step;
        ++k;
        if (k == target) {
            x = x1;
            break;
        }
        const unsigned long long bx = double_bits(x), b1 = double_bits(x1);
        const int ex = static_cast<int>((bx >> 52) & 0x7FF), e1 = static_cast<int>((b1 >> 52) & 0x7FF);
        // same sign, same normal binade, x moving (|d| >= one grid step)
        if (ex == e1 && ex != 0 && ex != 0x7FF && (bx >> 63) == (b1 >> 63) && bx != b1) {
            const double d = x1 - x;     // exact: same binade
            const double e = step - d;   // the rounding error of x + step, exact
            const long long M1 = static_cast<long long>(b1 & 0xFFFFFFFFFFFFFull) | (1ll << 52);
            const long long M0 = static_cast<long long>(bx & 0xFFFFFFFFFFFFFull) | (1ll << 52);
            const long long D = M1 - M0;  // increment in grid units (significand steps)
            const double u = bits_double(static_cast<unsigned long long>(ex - 52) << 52);  // the grid
            // a tie (|e| == u/2) rounds by the parity of x: not a fixed increment
            if (!(e == 0.5 * u || e == -0.5 * u) && D != 0) {
                // steps that stay strictly inside the binade, with a margin of two
                // increments for the exact sum before rounding
                const long long room = D > 0 ? (1ll << 53) - 1 - M1 : M1 - (1ll << 52);
                const long long ad = D > 0 ? D : -D;
                // a lower bound of room / ad - 2 in FP32 (conversions and the
                // quotient are within 3 * 2^-24 relative; the factor 1 - 2^-20
                // keeps it below the exact quotient): a shorter jump only costs
                // another iteration, while a 64-bit integer division costs
                // hundreds of dependent instructions on the device
                long long m = static_cast<long long>(static_cast<float>(room) / static_cast<float>(ad) *
                                                     0.99999904632568359375f) - 2;
                if (m > static_cast<long long>(target - k)) m = target - k;
                if (m > 0) {
                    const unsigned long long bm =
                        (b1 & ~0xFFFFFFFFFFFFFull) |
                        (static_cast<unsigned long long>(M1 + m * D) & 0xFFFFFFFFFFFFFull);
                    x = bits_double(bm);
                    k += static_cast<int>(m);
                    continue;
                }
            }
        }
        x = x1;
    }
    w->x = x;
    w->k = k;
}

// The reference's decision for sample k (x accumulated from begin, k steps).
CTR_HD bool acc_inside(double begin, double step, int n, int k)
{
    double x = begin;
    for (int j = 0; j < k; ++j) x += step;
    return x >= 0.0 && x <= static_cast<double>(n - 1);
}

// 32.32 fixed point -> float (integer conversions only; relative error ~1e-7).
CTR_HD float fix_to_float(long long X)
{
    return static_cast<float>(static_cast<int>(X >> 32)) +
           static_cast<float>(static_cast<unsigned>(X) >> 8) * 5.9604644775390625e-8f;
}

// Column ray in band rows [b0, b1]: the samples ix in [lo, hi] whose row
// floor(Y(ix)) lies in the band, Y(ix) = X0 + ix * S (monotone in ix), as
// [*ia, *ib] (empty when *ib < *ia).  The band's first sample and the first
// sample past it are each the first index satisfying a monotone predicate,
// found from an FP32 estimate settled on the integer positions (bisection
// where the estimate is far off: a step near 0).
CTR_HD void col_range(long long X0, long long S, int b0, int b1, int lo, int hi, int* ia, int* ib)
{
    const long long B0 = static_cast<long long>(b0) << 32, B1 = static_cast<long long>(b1 + 1) << 32;
    auto Y = [&](int ix) { return X0 + static_cast<long long>(ix) * S; };
    if (S == 0) {
        const bool in = X0 >= B0 && X0 < B1;
        *ia = in ? lo : 1;
        *ib = in ? hi : 0;
        return;
    }
    const float y0 = fix_to_float(X0), inv = 1.0f / fix_to_float(S);
    const bool up = S > 0;
    // first ix in [lo, hi + 1] with (up ? Y >= T : Y < T)
    auto first = [&](long long T, float tb) -> int {
        auto pred = [&](int ix) { return up ? Y(ix) >= T : Y(ix) < T; };
        const float t = (tb - y0) * inv;  // real crossing
        float e = up ? std::ceil(t) : std::floor(t) + 1.0f;
        e = e < static_cast<float>(lo) ? static_cast<float>(lo)
                                       : (e > static_cast<float>(hi + 1) ? static_cast<float>(hi + 1) : e);
        int k = static_cast<int>(e);
        for (int it = 0; it < 4 && k > lo && pred(k - 1); ++it) --k;
        for (int it = 0; it < 4 && k <= hi && !pred(k); ++it) ++k;
        if ((k == lo || !pred(k - 1)) && (k > hi || pred(k))) return k;
        int l = lo, h = hi + 1;
        while (l < h) {
            const int m = (l + h) >> 1;
            if (pred(m)) h = m;
            else l = m + 1;
        }
        return l;
    };
    const float fb0 = static_cast<float>(b0), fb1 = static_cast<float>(b1 + 1);
    *ia = up ? first(B0, fb0) : first(B1, fb1);
    *ib = (up ? first(B1, fb1) : first(B0, fb0)) - 1;
}

// The reference's own rule for a ray the integer path could not settle: x
// accumulated sample by sample in FP64 (x += step, src/fp_par_2d.cc:236-249),
// sample k used iff 0 <= x <= n-1.  The 32.32 line is anchored at the
// smallest-x valid sample, so X >= 0 on every valid sample.  Rare (ties at the
// image border), so its n FP64 additions cost nothing overall.
CTR_HD void ray_fp64_n(double begin, double step, int n, int ext, long long* X0, long long* Sout,
                       int* k0o, int* k1o)
{
    const double lim = static_cast<double>(ext - 1);
    int k0 = n, k1 = -1;
    double x = begin;
    for (int k = 0; k < n; ++k) {
        if (x >= 0.0 && x <= lim) {
            if (k0 == n) k0 = k;
            k1 = k;
        }
        x += step;
    }
    long long S = 0, X = 0;
    if (k0 <= k1) {
        S = std::fabs(step) < 1048576.0 ? std::llrint(step * kFix32) : 0;
        const int ka = step < 0.0 ? k1 : k0;  // smallest x
        const double xa = std::fma(static_cast<double>(ka), step, begin);
        X = std::llrint((xa > 0.0 ? xa : 0.0) * kFix32) - static_cast<long long>(ka) * S;
    } else {
        k0 = 1;
        k1 = 0;
    }
    *X0 = X;
    *Sout = S;
    *k0o = k0;
    *k1o = k1;
}

CTR_HD void ray_fp64(double begin, double step, int n, long long* X0, long long* Sout, int* k0o,
                     int* k1o)
{
    ray_fp64_n(begin, step, n, n, X0, Sout, k0o, k1o);
}

// The exact range [*k0, *k1] (empty: *k1 < *k0) of samples k < n of a line
// whose FP64 running position (begin + step + ... , k additions) lies in
// [0, ext-1], with the line's 32.32 fixed-point form: fixed point where that is
// certain, the accumulation itself (acc_advance) for the up to two ambiguous
// samples at each end, the plain FP64 walk otherwise.  The position is
// monotone in k, so the range is contiguous.
CTR_HD void axis_range(double begin, double step, int n, int ext, long long* X0, long long* S, int* k0,
                       int* k1)
{
    if (ray_fixed_n(begin, step, n, ext, X0, S, k0, k1)) return;
    int amb[4], namb = 0, c0, c1;
    if (ray_split_n(begin, step, n, ext, X0, S, &c0, &c1, amb, &namb)) {
        for (int a = 1; a < namb; ++a)
            for (int b = a; b > 0 && amb[b] < amb[b - 1]; --b) {
                const int t = amb[b];
                amb[b] = amb[b - 1];
                amb[b - 1] = t;
            }
        bool in[4] = {false, false, false, false};
        AccWalk w{begin, 0};
        for (int a = 0; a < namb; ++a) {
            acc_advance(&w, step, amb[a]);
            in[a] = w.x >= 0.0 && w.x <= static_cast<double>(ext - 1);
        }
        int lo = c0, hi = c1;
        for (int k = c0 - 1; k >= c0 - 2; --k) {  // contiguous: stop at the first outside
            bool ok = false;
            for (int a = 0; a < namb; ++a)
                if (amb[a] == k) ok = in[a];
            if (!ok) break;
            lo = k;
        }
        for (int k = c1 + 1; k <= c1 + 2; ++k) {
            bool ok = false;
            for (int a = 0; a < namb; ++a)
                if (amb[a] == k) ok = in[a];
            if (!ok) break;
            hi = k;
        }
        *k0 = lo;
        *k1 = hi;
        return;
    }
    ray_fp64_n(begin, step, n, ext, X0, S, k0, k1);
}

}  // namespace ctr
