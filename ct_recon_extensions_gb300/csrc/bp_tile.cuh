// Device side of the FP32 pixel-driven backprojectors, shared by the
// single-geometry entry points (bp.cu) and the batched plan (batch.cu): view
// parameters, detector windows, tile-relative channel positions, the fast
// interior and exact edge tap paths, and the tile bodies of the forward
// operator.  Everything here has internal linkage per file.
//
// Channel positions are taken relative to each tile's reference pixel (the
// pixel nearest the tile centre), whose position is computed per (tile, view)
// in FP64 from the caller's tables.  The FP32 part then only adds offsets
// within the tile, so its rounding is that of a small quantity:
//   parallel: s = s(ref) + ox cos t / ds + oy sin t / ds, slopes from the
//             caller's FP64 x cos t / y sin t tables;
//   fan:      gamma = gamma(ref) + atan(tau), tau = (ox a + oy b) /
//             (1 + ox b - oy a), where (a, b) = (A, B) / R^2 and (A, B) is the
//             source-to-reference-pixel vector in the view's frame (R its
//             length), and the distance weight 1/(d^2 + r^2) =
//             (1/R^2) / (dn^2 + n^2) with n = ox a + oy b, dn = 1 + ox b - oy a.
// (ox, oy) is the pixel's offset from the reference pixel in mm.  Positions
// are stored as sigma = s - (lo + kc + 1/2): lo is the tile's detector window
// start and kc its centre, so |sigma| <= W/2 and the staged pairs hold
// (p[j] - (j - kc - 1/2) d[j], d[j]), d[j] = p[j+1] - p[j]; a tap is one
// 8-byte shared load at j = round(sigma) + kc and one FMA, q + sigma d.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>

#include "ctr_async.cuh"
#include "ctr_common.cuh"
#include "sk_split.h"

namespace ctr {
namespace {

constexpr int kBpThreads = 256;
constexpr int kTileX = 32;
// Rows per thread of the single-geometry kernels (tile 32 x 64); the batched
// plan's autotuner also runs 2 and 4.
constexpr int kRowsPerThread = 8;
constexpr int kTileY = (kBpThreads / 32) * kRowsPerThread;
constexpr int kViewBlock = 16;

enum class Geo { kFan, kPar };

// Fan relative-position variants (gen_atan_poly.py): a tile takes the last
// (smallest) range that covers |tau| on all its pixels.
// |t| <= 0.3: atan degree 4 (8.5e-10); |t| <= 0.12: degree 3 (3.6e-11);
// |t| <= 0.06: degree 2 (2.1e-10)
constexpr int kRelVariants = 3;
__host__ __device__ constexpr float rel_tmax(int v) { return v == 0 ? 0.3f : v == 1 ? 0.12f : 0.06f; }
constexpr int kRelAtanDeg[kRelVariants] = {4, 3, 2};
constexpr double kRelAtan[3][5] = {{9.99999999147148877e-01, -3.33332854976151782e-01, 1.99956912895000311e-01, -1.41487832354163345e-01, 9.29816211336887688e-02},
    {9.99999999963666064e-01, -3.33333252438835770e-01, 1.99971830243045878e-01, -1.39709592103805486e-01, 0.00000000000000000e+00},
    {9.99999999792751670e-01, -3.33332296470573552e-01, 1.99231096240648553e-01, 0.00000000000000000e+00, 0.00000000000000000e+00}};
// atan(j/16) for j = 0..kAtanTab-1 (filled on the host): the reference ray's
// angle is atan(j/16) + atan(delta) with |delta| <= 1/32.
constexpr int kAtanTab = 17;

// Per-launch constants of the FP32 tile kernels.
struct TileConst {
    int ns, na, nx, ny;
    int W;                 // staged window length (channels)
    int kc;                // window centre (W / 2)
    int WB;                // bulk-copy box (elements) per view: >= W + 4, multiple of 4
    int WS;                // shared slot stride per view: WB rounded up to 128 bytes
    float cents;           // (ns-1)/2 + offset_s
    float nsm1;            // ns - 1
    float dso, K;          // fan, FP32: source distance, dsd/ds (window corners, absolute path)
    float scale;           // applied once to the final sum
    int fx_bits;           // adjoint: fixed-point bits of a unit tap (see bp.cu)
    double orbit_start, orbit;  // parallel: view angle = orbit_start + ia*orbit
    double inv_ds;         // parallel: 1/ds
    double inv_dx, inv_dy; // parallel: 1/dx, 1/dy
    double centx, centy, dx, dy;  // pixel grid (centres: parallel)
    float dxf, dyf;        // pixel pitch in FP32
    double ds_d, cents_d, dso_d, dsd_d, K_d;  // FP64 geometry
    float apoly[kRelVariants][5];  // fan: (dsd/ds) atan(t)/t in powers of t^2
    double atab[kAtanTab];
    long long total4;      // sinogram elements of the launch, rounded down to 4
    size_t proj_stride, img_stride;
};

// Sets the window length and everything derived from it.
inline void set_window(TileConst& c, int W)
{
    c.W = W;
    c.kc = W / 2;
    c.WB = (W + 4 + 3) / 4 * 4;
    c.WS = (c.WB + 31) / 32 * 32;
}

// Host: the fan's relative-position tables (scaled by dsd/ds where noted).
inline void fill_fan_tables(TileConst& c, double dsd, double ds)
{
    c.K_d = dsd / ds;
    for (int v = 0; v < kRelVariants; ++v)
        for (int k = 0; k < 5; ++k) c.apoly[v][k] = static_cast<float>(kRelAtan[v][k] * c.K_d);
    for (int j = 0; j < kAtanTab; ++j) c.atab[j] = std::atan(j / 16.0);
}

// FP32 channel positions near a detector end are within ~1e-3 channels of the
// reference's FP64 value on the absolute path (s up to ~2e3, plus atan2f
// error) and far closer on the relative paths.  Within kEdgeEps of an end the
// inclusion decision is recomputed in FP64 from the caller's tables.
constexpr float kEdgeEps = 2e-3f;

// round(x) for |x| < 2^22: bits(x + kMagic) - kMagicBits (round to nearest even).
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr unsigned kMagicBits = 0x4B400000u;

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float2 lds_f2(unsigned addr)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

__device__ __forceinline__ void red_shared_u32(unsigned addr, unsigned v)
{
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// ---- per-(tile, view) records ---------------------------------------------

// Modes of a (tile, view): below kModeFastBase, kModeSkip, kModeEdgeAbs or
// kModeEdgeRel + the fan variant; a fast view (every tap on the detector and
// inside the window, relative position) keeps, in place of its mode, a
// shared address base (a multiple of 4, at least kModeFastBase) with the
// fan's variant in the low two bits.
constexpr int kModeSkip = 1;     // the tile projects entirely off the detector
constexpr int kModeEdgeAbs = 2;  // fan only: absolute FP32 position (tiles the
                                 // relative form does not cover)
constexpr int kModeEdgeRel = 4;  // relative position, per-pixel inclusion test
constexpr int kModeFastBase = 8;

// The fields the fast path reads, one 16-byte shared load.
struct __align__(16) FastRec {
    float p0, p1;  // parallel: cos t/ds, sin t/ds; fan relative: a, b; fan
                   // absolute: sin b, cos b
    float cen;     // position of the reference pixel less (lo + kc + 1/2)
    int mode;      // kModeSkip / kModeEdgeAbs / kModeEdgeRel + variant, or a fast-path base
};
// The rest of a record (kept in a second array: 24 bytes of shared memory a view).
struct ViewAux {
    float e;       // fan relative: 1/R^2 (folded into the staged pairs); else 1
    int lo;        // first staged channel
};
struct ViewRec : FastRec {
    float e;
    int lo;
};
constexpr size_t kViewBytes = sizeof(FastRec) + sizeof(ViewAux);

__device__ __forceinline__ FastRec load_fast(const FastRec* v)
{
    const float4 f = *reinterpret_cast<const float4*>(v);
    return FastRec{f.x, f.y, f.z, __float_as_int(f.w)};
}
__device__ __forceinline__ void store_view(FastRec* vf, ViewAux* va, int i, const ViewRec& P)
{
    vf[i] = FastRec{P.p0, P.p1, P.cen, P.mode};
    va[i] = ViewAux{P.e, P.lo};
}

__device__ __forceinline__ bool mode_fast(int m) { return static_cast<unsigned>(m) >= kModeFastBase; }
__device__ __forceinline__ bool mode_edge_rel(int m) { return (m & ~3) == kModeEdgeRel; }
__device__ __forceinline__ int mode_variant(int m) { return m & 3; }

// Tile geometry shared by the forward and the adjoint: origin, reference
// pixel and the FP32 corners (absolute, for the window) and corner offsets.
struct TileBox {
    int tx0, ty0, ixm, iym;
    float x0, x1, y0, y1;      // absolute corner coordinates (mm)
    float ox0, ox1, oy0, oy1;  // corner offsets from the reference pixel (mm)
};

template <Geo G>
__device__ __forceinline__ double pix_x(const double* __restrict__ t0, int ix, const TileConst& c)
{
    if constexpr (G == Geo::kFan) return t0[ix];
    else return (ix - c.centx) * c.dx;
}
template <Geo G>
__device__ __forceinline__ double pix_y(const double* __restrict__ t1, int iy, const TileConst& c)
{
    if constexpr (G == Geo::kFan) return t1[iy];
    else return (c.centy - iy) * c.dy;
}
// Offsets of a pixel from the tile's reference pixel, rounded once to FP32.
// (Fan: from the caller's FP64 position tables; parallel: the pixel pitch
// times a small integer, in FP32.)
template <Geo G>
__device__ __forceinline__ float off_x(const double* __restrict__ t0, int ix, int ixm, const TileConst& c)
{
    if constexpr (G == Geo::kFan) return static_cast<float>(t0[ix] - t0[ixm]);
    else return static_cast<float>(ix - ixm) * c.dxf;
}
template <Geo G>
__device__ __forceinline__ float off_y(const double* __restrict__ t1, int iy, int iym, const TileConst& c)
{
    if constexpr (G == Geo::kFan) return static_cast<float>(t1[iy] - t1[iym]);
    else return static_cast<float>(iym - iy) * c.dyf;
}

template <Geo G>
__device__ __forceinline__ TileBox tile_box(const double* __restrict__ t0, const double* __restrict__ t1,
                                            int tile_x, int tile_y, int tile_h, const TileConst& c)
{
    TileBox B;
    B.tx0 = tile_x * kTileX;
    B.ty0 = tile_y * tile_h;
    B.ixm = min(B.tx0 + kTileX / 2, c.nx - 1);
    B.iym = min(B.ty0 + tile_h / 2, c.ny - 1);
    const int ix1 = min(B.tx0 + kTileX - 1, c.nx - 1), iy1 = min(B.ty0 + tile_h - 1, c.ny - 1);
    B.x0 = static_cast<float>(pix_x<G>(t0, B.tx0, c));
    B.x1 = static_cast<float>(pix_x<G>(t0, ix1, c));
    B.y0 = static_cast<float>(pix_y<G>(t1, B.ty0, c));
    B.y1 = static_cast<float>(pix_y<G>(t1, iy1, c));
    B.ox0 = off_x<G>(t0, B.tx0, B.ixm, c);
    B.ox1 = off_x<G>(t0, ix1, B.ixm, c);
    B.oy0 = off_y<G>(t1, B.ty0, B.iym, c);
    B.oy1 = off_y<G>(t1, iy1, B.iym, c);
    return B;
}

// Absolute FP32 channel position of pixel (x, y) and the fan distance weight
// 1/(d^2 + r^2); vp = (sin b, cos b) (fan) or (cos t/ds, sin t/ds) (parallel).
// Used for detector windows (tile corners) and the fan's absolute edge path.
template <Geo G>
__device__ __forceinline__ float channel_abs(float x, float y, float2 vp, const TileConst& c, float* w)
{
    if constexpr (G == Geo::kFan) {
        const float d = fmaf(-y, vp.y, fmaf(x, vp.x, c.dso));
        const float r = fmaf(x, vp.y, y * vp.x);
        *w = rcp_approx(fmaf(d, d, r * r));
        return fmaf(atan2f(r, d), c.K, c.cents);
    } else {
        *w = 1.0f;
        return fmaf(y, vp.y, fmaf(x, vp.x, c.cents));
    }
}

// The reference's FP64 channel position (src/bp_fan_2d.cc:66-69,
// src/bp_par_2d.cc:70) from the caller's tables: t0/t1/t2 are xpos/ypos/
// sincostbl (fan) or xcos/ysin (parallel).
template <Geo G>
__device__ __noinline__ double channel_exact(int ix, int iy, int ia, const double* __restrict__ t0,
                                             const double* __restrict__ t1,
                                             const double* __restrict__ t2, const TileConst& c)
{
    if constexpr (G == Geo::kFan) {
        const double x = t0[ix], y = t1[iy], sb = t2[2 * ia], cb = t2[2 * ia + 1];
        const double d = __dadd_rn(c.dso_d, __dadd_rn(__dmul_rn(x, sb), -__dmul_rn(y, cb)));
        const double r = __dadd_rn(__dmul_rn(x, cb), __dmul_rn(y, sb));
        return __dadd_rn(__ddiv_rn(__dmul_rn(atan2(r, d), c.dsd_d), c.ds_d), c.cents_d);
    } else {
        const double xc = t0[static_cast<size_t>(ix) * c.na + ia];
        const double ys = t1[static_cast<size_t>(iy) * c.na + ia];
        return __dadd_rn(__ddiv_rn(__dadd_rn(xc, ys), c.ds_d), c.cents_d);
    }
}

// Tiles whose channel range lies farther than this outside [0, ns-1] project
// entirely off the detector (FP32 corner positions are within ~3e-4 channels).
constexpr float kSkipEps = 1e-2f;

// Detector window [lo, lo+W) that covers every tap of the tile for one view;
// *interior is set when every pixel of the tile projects at least one channel
// inside the detector (no inclusion test needed) and the window fits; *off
// when every pixel projects outside the detector (the view adds nothing).
// The channel position over a convex tile is extreme at its corners (affine
// for the parallel beam; for the fan the ray angle is).
template <Geo G>
__device__ int window_start(float2 vp, const TileBox& B, const TileConst& c, bool* interior, bool* off)
{
    float smin = FLT_MAX, smax = -FLT_MAX;
    bool full = false;
    const float xs[2] = {B.x0, B.x1}, ys[2] = {B.y0, B.y1};
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if constexpr (G == Geo::kFan) {
                const float d = fmaf(-ys[j], vp.y, fmaf(xs[i], vp.x, c.dso));
                if (d <= 0.0f) full = true;
            }
            float w;
            const float s = channel_abs<G>(xs[i], ys[j], vp, c, &w);
            smin = fminf(smin, s);
            smax = fmaxf(smax, s);
        }
    }
    *interior = false;
    *off = false;
    if (full || !(smin == smin) || !(smax == smax)) return -1;
    *off = smax < -kSkipEps || smin > c.nsm1 + kSkipEps;
    int lo = static_cast<int>(floorf(smin)) - 2;
    int hi = static_cast<int>(floorf(smax)) + 3;
    const bool fits = hi - lo + 1 <= c.W;
    *interior = fits && smin >= 1.0f && smax <= c.nsm1 - 1.0f;
    lo = max(lo, -1);
    hi = min(hi, c.ns);
    if (hi - lo + 1 > c.W && lo <= c.ns && hi >= -1) raise_flag(kFlagWindowOverflow);
    return min(lo, c.ns);
}

// FP64 1/x from the FP32 reciprocal and one Newton step (relative error
// ~1e-14 for x within FP32 range).
__device__ __forceinline__ double rcp_refined(double x)
{
    const double r = static_cast<double>(__frcp_rn(static_cast<float>(x)));
    return fma(r, fma(-x, r, 1.0), r);
}

// atan(t) for |t| <= (kAtanTab - 1/2)/16 in FP64: the table value at the
// nearest sixteenth, plus atan(delta) with delta = (t - t_j)/(1 + t t_j),
// |delta| <= 1/32, as delta - delta^3/3 + delta^5/5 (the next term is below
// 5e-12); the cubic and quintic terms (below 1.1e-5) are formed in FP32.
__device__ __forceinline__ double atan_ref(double t, const TileConst& c)
{
    const double q = rint(t * 16.0);
    const double tq = q * 0.0625;
    const double delta = (t - tq) * rcp_refined(fma(t, tq, 1.0));
    const float df = static_cast<float>(delta), d2 = df * df;
    const float corr = df * d2 * fmaf(d2, 0.2f, -1.0f / 3.0f);
    const int j = static_cast<int>(fabs(q));
    const double base = q < 0.0 ? -c.atab[j] : c.atab[j];
    return base + (delta + static_cast<double>(corr));
}

// Per-view parameters, window and path for one tile (thread-local).
template <Geo G>
__device__ ViewRec view_setup(const double* __restrict__ t0, const double* __restrict__ t1,
                              const double* __restrict__ t2, int ia, const TileBox& B,
                              const TileConst& c)
{
    ViewRec P;
    bool inner, off;
    if constexpr (G == Geo::kPar) {
        // slopes from the caller's FP64 tables (differences of neighbouring
        // pixels; the tables are x cos t and y sin t), reference position in
        // FP64 (src/bp_par_2d.cc:70): FP32 then rounds only in-tile offsets
        const size_t na = static_cast<size_t>(c.na);
        const int ixn = B.ixm + 1 < c.nx ? B.ixm + 1 : B.ixm - 1;
        const int iyn = B.iym + 1 < c.ny ? B.iym + 1 : B.iym - 1;
        const double xc = t0[B.ixm * na + ia], ys = t1[B.iym * na + ia];
        double cs = (c.nx > 1) ? (t0[ixn * na + ia] - xc) * c.inv_dx * (ixn > B.ixm ? 1.0 : -1.0) : 0.0;
        double sn = (c.ny > 1) ? (ys - t1[iyn * na + ia]) * c.inv_dy * (iyn > B.iym ? 1.0 : -1.0) : 0.0;
        if (c.nx == 1 || c.ny == 1) {
            // a one-pixel-wide image has no neighbour: use the view angle
            double sa, ca;
            ::sincos(c.orbit_start + ia * c.orbit, &sa, &ca);
            if (c.nx == 1) cs = ca;
            if (c.ny == 1) sn = sa;
        }
        P.p0 = static_cast<float>(cs * c.inv_ds);
        P.p1 = static_cast<float>(sn * c.inv_ds);
        P.lo = window_start<G>(make_float2(P.p0, P.p1), B, c, &inner, &off);
        P.cen = static_cast<float>((xc + ys) * c.inv_ds + c.cents_d - (P.lo + c.kc + 0.5));
        P.e = 1.0f;
        P.mode = inner ? kModeFastBase : (off ? kModeSkip : kModeEdgeRel);
    } else {
        const double sb = t2[2 * ia], cb = t2[2 * ia + 1];
        const double X = t0[B.ixm], Y = t1[B.iym];
        P.lo = window_start<G>(make_float2(static_cast<float>(sb), static_cast<float>(cb)), B, c, &inner, &off);
        // source-to-reference-pixel vector in the view's frame
        const double A = fma(c.dso_d, cb, -Y), Bv = fma(c.dso_d, sb, X);
        const double d0 = fma(A, cb, Bv * sb), r0 = fma(Bv, cb, -(A * sb));
        const double R2 = fma(A, A, Bv * Bv);
        bool rel = d0 > 0.0 && R2 > 0.0 && fabs(r0) <= (kAtanTab - 0.5) / 16.0 * d0;
        int v = 0;
        if (rel) {
            const double eR = rcp_refined(R2);
            P.p0 = static_cast<float>(A * eR);
            P.p1 = static_cast<float>(Bv * eR);
            P.e = static_cast<float>(eR);
            // largest |tau| over the tile: at a corner (the angle seen from the
            // source is monotone along each edge of the convex tile)
            float tmax = 0.0f;
            const float oxs[2] = {B.ox0, B.ox1}, oys[2] = {B.oy0, B.oy1};
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const float n = fmaf(oys[k], P.p1, oxs[i] * P.p0);
                    const float dn = fmaf(-oys[k], P.p0, fmaf(oxs[i], P.p1, 1.0f));
                    if (!(dn > 0.0f)) rel = false;
                    tmax = fmaxf(tmax, fabsf(n) / dn);
                }
            v = -1;
#pragma unroll
            for (int k = 0; k < kRelVariants; ++k)
                if (tmax <= rel_tmax(k)) v = k;
            if (v < 0) rel = false;
            if (rel) {
                const double g0 = atan_ref(r0 * rcp_refined(d0), c);
                P.cen = static_cast<float>(fma(g0, c.K_d, c.cents_d - (P.lo + c.kc + 0.5)));
            }
        }
        if (!rel) {
            P.p0 = static_cast<float>(sb);
            P.p1 = static_cast<float>(cb);
            P.cen = 0.0f;
            P.e = 1.0f;
        }
        P.mode = off ? kModeSkip : (rel ? (inner ? kModeFastBase : kModeEdgeRel) + v : kModeEdgeAbs);
    }
    return P;
}

// ---- channel positions (bit-identical wherever they are computed) ----------
// Every operation below is an explicit round-to-nearest intrinsic, so the
// forward kernels and the adjoint compute the same position for a
// (pixel, view): the adjoint is then the exact transpose of the forward.

// Parallel beam: sigma = cen + ox p0 + oy p1 (x part once per column).
__device__ __forceinline__ float par_xpart(float ox, const FastRec& P) { return __fmaf_rn(ox, P.p0, P.cen); }
__device__ __forceinline__ float par_sigma(float xs, float oy, const FastRec& P) { return __fmaf_rn(oy, P.p1, xs); }

// Fan: x part (ox a, 1 + ox b) once per column; then per pixel
// tau = n / dn, n = ox a + oy b, dn = 1 + ox b - oy a, sigma = cen +
// (dsd/ds) atan(tau), weight w = 1/(dn^2 + n^2) (the view's 1/R^2 is in the
// staged pairs).
struct FanX {
    float n, d;
};
__device__ __forceinline__ FanX fan_xpart(float ox, const FastRec& P)
{
    return FanX{__fmul_rn(ox, P.p0), __fmaf_rn(ox, P.p1, 1.0f)};
}
template <int V>
__device__ __forceinline__ float fan_sigma(FanX X, float oy, const FastRec& P, const TileConst& c, float* w)
{
    constexpr int da = kRelAtanDeg[V];
    const float n = __fmaf_rn(oy, P.p1, X.n);
    const float dn = __fmaf_rn(-oy, P.p0, X.d);
    const float t = __fmul_rn(n, rcp_approx(dn));
    const float z = __fmul_rn(t, t);
    float p = c.apoly[V][da];
#pragma unroll
    for (int k = da - 1; k >= 0; --k) p = __fmaf_rn(z, p, c.apoly[V][k]);
    *w = rcp_approx(__fmaf_rn(dn, dn, __fmul_rn(n, n)));
    return __fmaf_rn(t, p, P.cen);
}

// round(sigma) as a float (exact).
__device__ __forceinline__ float round_sigma(float sig) { return __fadd_rn(__fadd_rn(sig, kMagic), -kMagic); }

// One tap on an edge view, relative position: inclusion decided as the
// reference does (0 <= s <= ns-1, in FP64 within kEdgeEps of an end); returns
// false when excluded, else the pair index j (in [0, W-2]) and *sig2, the
// position relative to the window centre used for the interpolation
// (q[j] + sig2 d[j]; the fraction beyond j is sig2 - (j - kc - 1/2)).
template <Geo G>
__device__ __forceinline__ bool edge_tap(float sig, int ix, int iy, int ia, int lo, const double* t0,
                                         const double* t1, const double* t2, const TileConst& c,
                                         int* j, float* sig2)
{
    const float s = __fadd_rn(sig, static_cast<float>(lo + c.kc) + 0.5f);  // absolute, FP32
    if (fabsf(s) < kEdgeEps || fabsf(s - c.nsm1) < kEdgeEps) {
        const double sd = channel_exact<G>(ix, iy, ia, t0, t1, t2, c);
        if (!(sd >= 0.0 && sd <= static_cast<double>(c.ns - 1))) return false;
        const double fd = floor(sd);
        *j = static_cast<int>(fd) - lo;
        *sig2 = static_cast<float>(sd - (lo + c.kc + 0.5));
    } else {
        if (!(s >= 0.0f && s <= c.nsm1)) return false;
        *j = static_cast<int>(round_sigma(sig)) + c.kc;
        *sig2 = sig;
    }
    if (*j < 0 || *j > c.W - 2) {
        *j = min(max(*j, 0), c.W - 2);
        *sig2 = fminf(fmaxf(*sig2, static_cast<float>(*j - c.kc) - 0.5f), static_cast<float>(*j - c.kc) + 0.5f);
    }
    return true;
}

// The same on an absolute FP32 position s (fan tiles the relative form does
// not cover).
template <Geo G>
__device__ __forceinline__ bool edge_tap_abs(float s, int ix, int iy, int ia, int lo, const double* t0,
                                             const double* t1, const double* t2, const TileConst& c,
                                             int* j, float* sig2)
{
    double sd;
    if (fabsf(s) < kEdgeEps || fabsf(s - c.nsm1) < kEdgeEps) {
        sd = channel_exact<G>(ix, iy, ia, t0, t1, t2, c);
        if (!(sd >= 0.0 && sd <= static_cast<double>(c.ns - 1))) return false;
    } else {
        if (!(s >= 0.0f && s <= c.nsm1)) return false;
        sd = static_cast<double>(s);
    }
    const double fd = floor(sd);
    *j = min(max(static_cast<int>(fd) - lo, 0), c.W - 2);
    *sig2 = static_cast<float>(fmin(fmax(sd - (lo + c.kc + 0.5), (*j - c.kc) - 0.5), (*j - c.kc) + 0.5));
    return true;
}

// Pair of staged window element k (channel lo + k): (q, d) scaled by e, with
// d = p[k+1] - p[k] and q = p[k] - (k - kc - 1/2) d.
__device__ __forceinline__ float2 make_pair(float p0, float p1, int k, int kc, float e)
{
    const float d = p1 - p0;
    const float q = fmaf(-(static_cast<float>(k - kc) - 0.5f), d, p0);
    return make_float2(q * e, d * e);
}

// ---- fast-path taps of the forward ------------------------------------------

// The fast-path taps of one view for a thread's R pixels (fan variant V):
// pixel r is at offsets (ox, oy[r]); base = the view's pair slot address
// plus 8 kc, less 8 kMagicBits.
// Rows are taken in pairs: the position arithmetic of rows r and r+1 runs as
// packed FP32 pairs (FFMA2 / FADD2 / FMUL2, each half rounded as the scalar
// operation, so positions are bit-identical to fan_sigma / par_sigma and the
// forward's and adjoint's taps agree), and so do the running sums (the fan's
// weighted add, the parallel beam's add): each half is the scalar update.
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// a - b per half (an FMA with -1: exact negation, one rounding).
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, dup2(-1.0f), a); }

// fan_sigma for two pixels (x parts xn, xd; y offsets o), with their weights.
template <int V>
__device__ __forceinline__ float2 fan_sigma2(float2 xn, float2 xd, float2 o, const FastRec& P,
                                             const TileConst& c, float2* w)
{
    constexpr int da = kRelAtanDeg[V];
    const float2 n = __ffma2_rn(o, dup2(P.p1), xn);
    const float2 dn = __ffma2_rn(o, dup2(-P.p0), xd);  // -oy p0 + d
    const float2 t = __fmul2_rn(n, make_float2(rcp_approx(dn.x), rcp_approx(dn.y)));
    const float2 z = __fmul2_rn(t, t);
    float2 pp = dup2(c.apoly[V][da]);
#pragma unroll
    for (int k = da - 1; k >= 0; --k) pp = __ffma2_rn(z, pp, dup2(c.apoly[V][k]));
    const float2 q = __ffma2_rn(dn, dn, __fmul2_rn(n, n));
    *w = make_float2(rcp_approx(q.x), rcp_approx(q.y));
    return __ffma2_rn(t, pp, dup2(P.cen));
}

template <Geo G, int V, int R>
__device__ __forceinline__ void fast_rows(float ox, const float (&oy)[R], const FastRec& P,
                                          const TileConst& c, unsigned base, float (&part)[R])
{
    static_assert(R % 2 == 0, "rows are taken in pairs");
    const float2 mag = dup2(kMagic);
    if constexpr (G == Geo::kFan) {
        const FanX X = fan_xpart(ox, P);
        const float2 xn = dup2(X.n), xd = dup2(X.d);
#pragma unroll
        for (int r = 0; r < R; r += 2) {
            float2 w;
            const float2 sig = fan_sigma2<V>(xn, xd, make_float2(oy[r], oy[r + 1]), P, c, &w);
            const float2 tm = __fadd2_rn(sig, mag);
            const float2 pa = lds_f2(base + 8u * __float_as_uint(tm.x));
            const float2 pb = lds_f2(base + 8u * __float_as_uint(tm.y));
            const float2 acc = __ffma2_rn(make_float2(fmaf(sig.x, pa.y, pa.x), fmaf(sig.y, pb.y, pb.x)), w,
                                          make_float2(part[r], part[r + 1]));
            part[r] = acc.x;
            part[r + 1] = acc.y;
        }
    } else {
        const float2 xs = dup2(par_xpart(ox, P)), p1 = dup2(P.p1);
#pragma unroll
        for (int r = 0; r < R; r += 2) {
            const float2 sig = __ffma2_rn(make_float2(oy[r], oy[r + 1]), p1, xs);  // par_sigma
            const float2 tm = __fadd2_rn(sig, mag);
            const float2 pa = lds_f2(base + 8u * __float_as_uint(tm.x));
            const float2 pb = lds_f2(base + 8u * __float_as_uint(tm.y));
            const float2 acc = __fadd2_rn(make_float2(part[r], part[r + 1]),
                                          make_float2(fmaf(sig.x, pa.y, pa.x), fmaf(sig.y, pb.y, pb.x)));
            part[r] = acc.x;
            part[r + 1] = acc.y;
        }
    }
}

// Edge-path taps of one view (pairs of the view at wj) for a thread's R
// pixels: column ixc at offset ox, rows iy0 + r (clamped to the image) at
// offsets oy[r].
template <int V, int R>
__device__ __forceinline__ void edge_rows_fan(FanX X, const float (&oy)[R], int ixc, int iy0, int ia,
                                              const FastRec& P, int lo, const float2* wj, const double* t0,
                                              const double* t1, const double* t2, const TileConst& c,
                                              float (&part)[R])
{
#pragma unroll
    for (int r = 0; r < R; ++r) {
        float w, sig2;
        int j;
        const float sig = fan_sigma<V>(X, oy[r], P, c, &w);
        if (edge_tap<Geo::kFan>(sig, ixc, min(iy0 + r, c.ny - 1), ia, lo, t0, t1, t2, c, &j, &sig2)) {
            const float2 pv = wj[j];
            part[r] = fmaf(fmaf(sig2, pv.y, pv.x), w, part[r]);
        }
    }
}

template <Geo G, int R>
__device__ __forceinline__ void edge_rows(float ox, const float (&oy)[R], int ixc, int iy0, int ia,
                                          const FastRec& P, int lo, const float2* wj, const double* t0,
                                          const double* t1, const double* t2, const TileConst& c,
                                          float (&part)[R])
{
    if constexpr (G == Geo::kFan) {
        if (P.mode == kModeEdgeAbs) {
            const float x = static_cast<float>(t0[ixc]);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int iyc = min(iy0 + r, c.ny - 1);
                float w, sig2;
                int j;
                const float s = channel_abs<G>(x, static_cast<float>(t1[iyc]), make_float2(P.p0, P.p1), c, &w);
                if (edge_tap_abs<G>(s, ixc, iyc, ia, lo, t0, t1, t2, c, &j, &sig2)) {
                    const float2 pv = wj[j];
                    part[r] = fmaf(fmaf(sig2, pv.y, pv.x), w, part[r]);
                }
            }
            return;
        }
        const FanX X = fan_xpart(ox, P);
        switch (mode_variant(P.mode)) {
            case 0: edge_rows_fan<0, R>(X, oy, ixc, iy0, ia, P, lo, wj, t0, t1, t2, c, part); break;
            case 1: edge_rows_fan<1, R>(X, oy, ixc, iy0, ia, P, lo, wj, t0, t1, t2, c, part); break;
            default: edge_rows_fan<2, R>(X, oy, ixc, iy0, ia, P, lo, wj, t0, t1, t2, c, part); break;
        }
    } else {
        const float xs = par_xpart(ox, P);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float sig2;
            int j;
            const float sig = par_sigma(xs, oy[r], P);
            if (edge_tap<G>(sig, ixc, min(iy0 + r, c.ny - 1), ia, lo, t0, t1, t2, c, &j, &sig2)) {
                const float2 pv = wj[j];
                part[r] += fmaf(sig2, pv.y, pv.x);
            }
        }
    }
}

// Fast-path taps of one view, dispatched on the fan variant.
template <Geo G, int R>
__device__ __forceinline__ void fast_view(float ox, const float (&oy)[R], const FastRec& P,
                                          const TileConst& c, float (&part)[R])
{
    const unsigned base = static_cast<unsigned>(P.mode) & ~3u;
    if constexpr (G == Geo::kFan) {
        switch (mode_variant(P.mode)) {
            case 0: fast_rows<G, 0, R>(ox, oy, P, c, base, part); break;
            case 1: fast_rows<G, 1, R>(ox, oy, P, c, base, part); break;
            default: fast_rows<G, 2, R>(ox, oy, P, c, base, part); break;
        }
    } else {
        fast_rows<G, 0, R>(ox, oy, P, c, base, part);
    }
}

// The fan variant shared by every view of n records at vr when all of them
// take the fast path, else -1 (warp-uniform; n <= 64).
__device__ __forceinline__ int block_variant(const FastRec* vr, int n)
{
    const int lane = threadIdx.x & 31;
    const int v0 = mode_variant(vr[0].mode);
    bool ok = true;
    for (int j = lane; j < n; j += 32) {
        const int m = vr[j].mode;
        ok = ok && mode_fast(m) && mode_variant(m) == v0;
    }
    return __all_sync(0xffffffffu, ok) ? v0 : -1;
}

// n views (records at vr) that all take the fast path with variant V: no
// per-view dispatch, two views per trip (same summation order as one by one).
template <Geo G, int V, int R>
__device__ __forceinline__ void fast_block(float ox, const float (&oy)[R], const FastRec* vr, int n,
                                           const TileConst& c, float (&part)[R])
{
    // a parallel-beam mode has no variant bits: it is the base itself
    constexpr unsigned kMask = G == Geo::kPar ? ~0u : ~3u;
    int j = 0;
    for (; j + 4 <= n; j += 4) {
        const FastRec F0 = load_fast(vr + j), F1 = load_fast(vr + j + 1);
        const FastRec F2 = load_fast(vr + j + 2), F3 = load_fast(vr + j + 3);
        fast_rows<G, V, R>(ox, oy, F0, c, static_cast<unsigned>(F0.mode) & kMask, part);
        fast_rows<G, V, R>(ox, oy, F1, c, static_cast<unsigned>(F1.mode) & kMask, part);
        fast_rows<G, V, R>(ox, oy, F2, c, static_cast<unsigned>(F2.mode) & kMask, part);
        fast_rows<G, V, R>(ox, oy, F3, c, static_cast<unsigned>(F3.mode) & kMask, part);
    }
    for (; j + 2 <= n; j += 2) {
        const FastRec F0 = load_fast(vr + j), F1 = load_fast(vr + j + 1);
        fast_rows<G, V, R>(ox, oy, F0, c, static_cast<unsigned>(F0.mode) & kMask, part);
        fast_rows<G, V, R>(ox, oy, F1, c, static_cast<unsigned>(F1.mode) & kMask, part);
    }
    if (j < n) {
        const FastRec F0 = load_fast(vr + j);
        fast_rows<G, V, R>(ox, oy, F0, c, static_cast<unsigned>(F0.mode) & kMask, part);
    }
}

// The taps of n views (records at vr and va, pairs of view j at w + j*W;
// view index ia0 + j) for a thread's R pixels.
template <Geo G, int R>
__device__ __forceinline__ void block_taps(float ox, const float (&oy)[R], int ixc, int iy0, int ia0,
                                           const FastRec* vr, const ViewAux* va, int n, const float2* w,
                                           const double* t0,
                                           const double* t1, const double* t2, const TileConst& c,
                                           float (&part)[R])
{
    if (n <= 0) return;
    const int v = block_variant(vr, n);
    if (v >= 0) {
        if constexpr (G == Geo::kFan) {
            switch (v) {
                case 0: fast_block<G, 0, R>(ox, oy, vr, n, c, part); break;
                case 1: fast_block<G, 1, R>(ox, oy, vr, n, c, part); break;
                default: fast_block<G, 2, R>(ox, oy, vr, n, c, part); break;
            }
        } else {
            fast_block<G, 0, R>(ox, oy, vr, n, c, part);
        }
        return;
    }
    for (int j = 0; j < n; ++j) {
        const FastRec F = load_fast(vr + j);
        if (mode_fast(F.mode)) fast_view<G, R>(ox, oy, F, c, part);
        else if (F.mode != kModeSkip)
            edge_rows<G, R>(ox, oy, ixc, iy0, ia0 + j, F, va[j].lo, w + j * c.W, t0, t1, t2, c, part);
    }
}

// A fast view's mode: the shared address of its pair slot plus 8 kc, less
// 8 kMagicBits, with the variant in the low bits (kModeEdgeRel + variant in
// the unlikely case that the address falls below kModeFastBase).
__device__ __forceinline__ int fast_mode(unsigned slot_addr, const TileConst& c, int mode)
{
    const unsigned base = slot_addr + 8u * static_cast<unsigned>(c.kc) - 8u * kMagicBits;
    const int v = mode_variant(mode);
    return base >= static_cast<unsigned>(kModeFastBase) ? static_cast<int>(base | static_cast<unsigned>(v))
                                                        : kModeEdgeRel + v;
}

// Forward FP32 tile kernel with cooperative (plain-load) staging: proj [na][ns]
// -> img [ny][nx] (batch in grid.z), tile 32 x kTileY.  t0/t1/t2: fan
// xpos/ypos/sincostbl, parallel xcos/ysin/unused.  Used where the bulk-copy
// kernel below does not apply (windows wider than its box, unaligned
// buffers); same positions and pairs, so the same sums up to the order of
// the view blocks.
template <Geo G>
__global__ void __launch_bounds__(kBpThreads, 2)
    bp_tile_f32_coop(const float* __restrict__ proj, float* __restrict__ img,
                     const double* __restrict__ t0, const double* __restrict__ t1,
                     const double* __restrict__ t2, const TileConst c)
{
    constexpr int R = kRowsPerThread;
    extern __shared__ __align__(16) float2 win[];  // [kViewBlock][W]
    __shared__ FastRec s_v[kViewBlock];
    __shared__ ViewAux s_a[kViewBlock];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileBox B = tile_box<G>(t0, t1, blockIdx.x, blockIdx.y, kTileY, c);
    const float* P_ = proj + blockIdx.z * c.proj_stride;
    const int ixc = min(B.tx0 + lane, c.nx - 1);
    const int iy0 = B.ty0 + warp * R;
    const float ox = off_x<G>(t0, ixc, B.ixm, c);
    float oy[R], acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        oy[r] = off_y<G>(t1, min(iy0 + r, c.ny - 1), B.iym, c);
        acc[r] = 0.0f;
    }
    const unsigned win_base = smem_u32(win);
    for (int v0 = 0; v0 < c.na; v0 += kViewBlock) {
        const int nv = min(kViewBlock, c.na - v0);
        if (threadIdx.x < nv) {
            ViewRec P = view_setup<G>(t0, t1, t2, v0 + threadIdx.x, B, c);
            if (mode_fast(P.mode)) P.mode = fast_mode(win_base + 8u * threadIdx.x * c.W, c, P.mode);
            store_view(s_v, s_a, threadIdx.x, P);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < nv * c.W; idx += kBpThreads) {
            const int j = idx / c.W, k = idx - j * c.W;
            const int g = s_a[j].lo + k;
            const float* row = P_ + static_cast<size_t>(v0 + j) * c.ns;
            const float p0 = (g >= 0 && g < c.ns) ? __ldg(row + g) : 0.0f;
            const float p1 = (g + 1 >= 0 && g + 1 < c.ns) ? __ldg(row + g + 1) : 0.0f;
            win[idx] = make_pair(p0, p1, k, c.kc, s_a[j].e);
        }
        __syncthreads();
        float part[R];
#pragma unroll
        for (int r = 0; r < R; ++r) part[r] = 0.0f;
        block_taps<G, R>(ox, oy, ixc, iy0, v0, s_v, s_a, nv, win, t0, t1, t2, c, part);
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] += part[r];
        __syncthreads();
    }
    float* I = img + blockIdx.z * c.img_stride;
    const int ix = B.tx0 + lane;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int iy = iy0 + r;
        if (ix < c.nx && iy < c.ny) I[static_cast<size_t>(iy) * c.nx + ix] = acc[r] * c.scale;
    }
}

// ---- bulk-copy-fed forward kernel ---------------------------------------------
//
// A CTA runs NG view groups of 256 threads on one 32 x (8 R) tile (each
// group takes its share of every block of NG*VB views; with two groups the
// partial sums are added in a fixed order at the end), and the detector
// windows reach shared memory through the TMA engine: one cp.async.bulk copy
// per view (16-byte aligned start in the flattened sinogram, a 128-byte
// aligned shared slot), issued two view blocks ahead into double-buffered raw
// slots, each block completed on its own mbarrier (waits are bounded and
// report kFlagWaitTimeout).  Once a slot has landed, the CTA rewrites it as
// pairs (make_pair), zero off the detector.
constexpr int kGroups = 2;
constexpr int kBlockViews = kGroups * kViewBlock;
constexpr int kTmaThreads = kGroups * kBpThreads;

// One tile (tile_x, tile_y) of item `item`, over its view blocks
// [b_begin, b_end) (b_end < 0: all); all NG*256 threads of the CTA call it.
// With `partial` null the scaled sums are stored to the image; otherwise the
// unscaled sums of this range go to partial[row * kTileX + column] of the tile.
// Re-entrant across calls of a persistent CTA: the mbarriers are
// (re)initialised here and every copy issued is waited on before returning.
// Returns false (uniformly) when a check or a bounded wait failed.
template <Geo G, int R = kRowsPerThread, int VB = kViewBlock, int NG = kGroups>
__device__ __forceinline__ bool tile_forward(const float* __restrict__ proj, float* __restrict__ img,
                                             const double* __restrict__ t0,
                                             const double* __restrict__ t1,
                                             const double* __restrict__ t2, const TileConst& c,
                                             int tile_x, int tile_y, int item, int b_begin = 0,
                                             int b_end = -1, float* __restrict__ partial = nullptr,
                                             const FastRec* __restrict__ rec = nullptr,
                                             const ViewAux* __restrict__ aux = nullptr)
{
    constexpr int kTY = (kBpThreads / 32) * R;  // tile height
    constexpr int kBV = NG * VB;                // views per staged block
    constexpr int kThreads = NG * kBpThreads;   // NG view groups of 256 threads
    // Dynamic shared memory, 128-byte aligned here: raw slots [2][kBV][WS]
    // (every slot stride a 128-byte multiple), pairs [2][kBV][W], then one
    // view record per view of the whole scan (FastRec array, then ViewAux).
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    unsigned char* smem = smem_dyn + ((128u - (smem_u32(smem_dyn) & 127u)) & 127u);
    float* raw = reinterpret_cast<float*>(smem);
    float2* pairs = reinterpret_cast<float2*>(smem + 2 * kBV * c.WS * sizeof(float));
    FastRec* views = reinterpret_cast<FastRec*>(pairs + 2 * kBV * c.W);
    ViewAux* vaux = reinterpret_cast<ViewAux*>(views + c.na);
    __shared__ __align__(8) unsigned long long s_bar[2];
    __shared__ int s_ok;

    const int tid = threadIdx.x;
    const int group = tid / kBpThreads;
    const int lt = tid - group * kBpThreads;
    const int lane = lt & 31, warp = lt >> 5;
    const TileBox B = tile_box<G>(t0, t1, tile_x, tile_y, kTY, c);
    const int nblocks = b_end < 0 ? (c.na + kBV - 1) / kBV : b_end;
    // double-buffer slots and barrier phases count from b_begin

    // Slot j of block b receives sinogram elements [gx, gx + WB) of the flattened
    // array (gx = window start rounded down to 4 elements, so the source is
    // 16-byte aligned), clipped to [0, total4) where total4 = total rounded down
    // to 4 elements; the conversion below reads the clipped-away elements from
    // global directly.
    auto slot_start = [&](int ia) -> long long {
        return (static_cast<long long>(item) * c.na + ia) * c.ns + vaux[ia].lo;
    };
    // Issued by warp 0, one lane per view (kBV <= 64: two rounds at most); lane 0
    // arms the barrier with the block's byte count (a warp sum) first.
    auto issue_block = [&](int b) {
        if (b >= nblocks) return;
        const int v0 = b * kBV;
        const int nv = min(kBV, c.na - v0);
        const int lb = b - b_begin;
        const unsigned bar = smem_u32(&s_bar[lb & 1]);
        float* slot = raw + (lb & 1) * kBV * c.WS;
        unsigned bytes = 0;
        for (int j = lane; j < nv; j += 32) {
            const long long gx = slot_start(v0 + j) & ~3ll;
            const long long g0 = max(gx, 0ll), g1 = min(gx + c.WB, c.total4);
            if (g1 > g0) bytes += static_cast<unsigned>((g1 - g0) * sizeof(float));
        }
        bytes = __reduce_add_sync(0xffffffffu, bytes);
        if (lane == 0) mbar_expect_tx(bar, bytes);
        __syncwarp();
        for (int j = lane; j < nv; j += 32) {
            const long long gx = slot_start(v0 + j) & ~3ll;
            const long long g0 = max(gx, 0ll), g1 = min(gx + c.WB, c.total4);
            if (g1 > g0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                bulk_load(smem_u32(slot + j * c.WS + (g0 - gx)), proj + g0,
                          static_cast<unsigned>((g1 - g0) * sizeof(float)), bar);
            }
        }
    };

    // a persistent CTA calls this tile after tile: every warp must be done
    // reading the previous tile's view records before they are overwritten
    __syncthreads();
    // per-view parameters, windows and paths of this tile for the whole scan;
    // a fast view keeps its pair slot's address base in place of its mode
    const unsigned pairs_base = smem_u32(pairs);
    const int ia_end = min(nblocks * kBV, c.na);
    for (int ia = b_begin * kBV + tid; ia < ia_end; ia += kThreads) {
        ViewRec P;
        if (rec) {  // a plan's record of this (tile, view)
            const size_t ti = (static_cast<size_t>(tile_y) * ((c.nx + kTileX - 1) / kTileX) + tile_x) * c.na + ia;
            const FastRec F = rec[ti];
            const ViewAux A = aux[ti];
            P.p0 = F.p0;
            P.p1 = F.p1;
            P.cen = F.cen;
            P.mode = F.mode;
            P.e = A.e;
            P.lo = A.lo;
        } else {
            P = view_setup<G>(t0, t1, t2, ia, B, c);
        }
        if (mode_fast(P.mode)) {
            const int slot = ((ia / kBV - b_begin) & 1) * kBV + ia % kBV;
            P.mode = fast_mode(pairs_base + 8u * static_cast<unsigned>(slot * c.W), c, P.mode);
        }
        store_view(views, vaux, ia, P);
    }
    if (tid == 0) {
        // every copy destination must be 128-byte aligned; check before issuing any
        const bool aligned = (smem_u32(raw) & 127u) == 0 && (c.WS * sizeof(float)) % 128 == 0;
        // the group reduction at the end writes R x kBpThreads floats into one
        // half of the pair buffer (kBV x W float2)
        const bool fits = NG == 1 || R * kBpThreads <= 2 * kBV * c.W;
        s_ok = aligned && fits;
        if (!aligned) raise_flag(kFlagMisaligned);
        if (!fits) raise_flag(kFlagWindowOverflow);
        mbar_init(smem_u32(&s_bar[0]), 1);
        mbar_init(smem_u32(&s_bar[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (!s_ok) return false;
    if (tid < 32) {
        issue_block(b_begin);
        issue_block(b_begin + 1);
    }

    const int ixc = min(B.tx0 + lane, c.nx - 1);
    const int iy0 = B.ty0 + warp * R;
    const float ox = off_x<G>(t0, ixc, B.ixm, c);
    float oy[R], acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        oy[r] = off_y<G>(t1, min(iy0 + r, c.ny - 1), B.iym, c);
        acc[r] = 0.0f;
    }

    const int wid = tid >> 5;  // warp of the CTA
    for (int b = b_begin; b < nblocks; ++b) {
        const int lb = b - b_begin;
        // every thread waits for block b's copies (bounded); a timeout is
        // reported and the block proceeds, so no thread is left at a barrier
        if (!mbar_wait_bounded(smem_u32(&s_bar[lb & 1]), (lb >> 1) & 1) && tid == 0)
            raise_flag(kFlagWaitTimeout);
        const int nv = min(kBV, c.na - b * kBV);
        const float* slot = raw + (lb & 1) * kBV * c.WS;
        float2* pb = pairs + (lb & 1) * kBV * c.W;
        // one warp per view: rewrite the raw window as pairs
        for (int j = wid; j < nv; j += kThreads / 32) {
            const long long st = slot_start(b * kBV + j);
            const int lo = vaux[b * kBV + j].lo;
            const float e = vaux[b * kBV + j].e;
            const float* src = slot + j * c.WS + static_cast<int>(st & 3ll);
            float2* dst = pb + j * c.W;
            if (lo >= 0 && lo + c.W < c.ns && st + c.W < c.total4) {
                // make_pair with (k - kc - 1/2) carried as a float (exact) and,
                // for the parallel beam, its unit scale left out
                float fk = static_cast<float>(lane - c.kc) - 0.5f;
                for (int k = lane; k < c.W; k += 32, fk += 32.0f) {
                    const float p0 = src[k], d = src[k + 1] - p0;
                    const float q = fmaf(-fk, d, p0);
                    dst[k] = G == Geo::kPar ? make_float2(q, d) : make_float2(q * e, d * e);
                }
            } else {  // a detector end or the array's ragged tail is in the window
                for (int k = lane; k < c.W; k += 32) {
                    auto at = [&](int gg, long long ii, const float* sp) -> float {
                        if (gg < 0 || gg >= c.ns) return 0.0f;  // off the detector
                        return ii < c.total4 ? *sp : __ldg(proj + ii);
                    };
                    dst[k] = make_pair(at(lo + k, st + k, src + k), at(lo + k + 1, st + k + 1, src + k + 1), k,
                                       c.kc, e);
                }
            }
        }
        __syncthreads();
        if (tid < 32) issue_block(b + 2);  // block b's raw slot has been consumed

        const int jb = group * VB;
        const int je = min(jb + VB, nv);
        float part[R];  // this block's partial sums (blocked summation)
#pragma unroll
        for (int r = 0; r < R; ++r) part[r] = 0.0f;
        block_taps<G, R>(ox, oy, ixc, iy0, b * kBV + jb, views + b * kBV + jb, vaux + b * kBV + jb, je - jb,
                         pb + jb * c.W, t0, t1, t2, c, part);
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] += part[r];
    }
    // with two groups, add the second group's sums to the first's, in that
    // order; the reduction uses the pairs buffer of the next-to-last block,
    // which every thread has finished reading before the last block's barrier
    // (or one never used)
    float* red = reinterpret_cast<float*>(pairs + ((nblocks - b_begin) & 1) * kBV * c.W);
    if constexpr (NG == 2) {
        if (group == 1) {
#pragma unroll
            for (int r = 0; r < R; ++r) red[r * kBpThreads + lt] = acc[r];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] += group == 0 ? red[r * kBpThreads + lt] : 0.0f;
    }
    if (group == 0) {
        if (partial) {
#pragma unroll
            for (int r = 0; r < R; ++r) partial[(warp * R + r) * kTileX + lane] = acc[r];
        } else {
            float* I = img + static_cast<size_t>(item) * c.img_stride;
            const int ix = B.tx0 + lane;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int iy = iy0 + r;
                if (ix < c.nx && iy < c.ny) I[static_cast<size_t>(iy) * c.nx + ix] = acc[r] * c.scale;
            }
        }
    }
    return true;
}

template <Geo G, int R, int MinBlocks, int VB, int NG>
__global__ void __launch_bounds__(NG * kBpThreads, MinBlocks)
    bp_tile_tma_f32(const float* __restrict__ proj, float* __restrict__ img,
                    const double* __restrict__ t0, const double* __restrict__ t1,
                    const double* __restrict__ t2, const TileConst c,
                    const FastRec* __restrict__ rec = nullptr, const ViewAux* __restrict__ aux = nullptr)
{
    grid_dep_wait();  // launched as a dependent of the kernel before it
    tile_forward<G, R, VB, NG>(proj, img, t0, t1, t2, c, blockIdx.x, blockIdx.y, blockIdx.z, 0, -1, nullptr,
                               rec, aux);
}

// A plan's per-(tile, view) records (tiles of 32 x kTileY, [tile][view], the
// mode before its pair-slot base): one thread each.
template <Geo G>
__global__ void __launch_bounds__(256)
    bp_view_records(const double* __restrict__ t0, const double* __restrict__ t1,
                    const double* __restrict__ t2, const TileConst c, int tiles_x, int tiles,
                    FastRec* __restrict__ rec, ViewAux* __restrict__ aux)
{
    const long long n = static_cast<long long>(tiles) * c.na;
    for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += gridDim.x * 256ll) {
        const int t = static_cast<int>(i / c.na), ia = static_cast<int>(i - static_cast<long long>(t) * c.na);
        const TileBox B = tile_box<G>(t0, t1, t % tiles_x, t / tiles_x, kTileY, c);
        store_view(rec, aux, static_cast<int>(i), view_setup<G>(t0, t1, t2, ia, B, c));
    }
}

// ---- stream-K split of small launches ----------------------------------------
//
// A launch with few tiles (a 512^2 image is 128 tiles of 32 x 64) leaves SMs
// idle when each CTA owns whole tiles.  Here the work is cut into units of
// (tile, block of NG*VB views), tiles outer, and CTA c of G takes the
// contiguous units [c*U/G, (c+1)*U/G): every SM gets the same number of view
// blocks.  A tile whose units span several CTAs gets one unscaled partial sum
// per CTA (segment) in `partial`; each CTA counts its segment in on the
// tile's counter, and the CTA that completes the count adds the segments in
// segment order, scales and stores the tile (deterministic).
struct SkConst {
    long long units;       // tiles x nb
    int nb;                // view blocks per tile
    int tiles_x, tiles_per_item;
    int maxseg;            // segments per tile, at most
    float* partial;        // [tiles][maxseg][kTileX x tile height]
    int* counter;          // [tiles], zero at launch; the CTA completing a tile resets it
    const FastRec* rec;    // a plan's per-(tile, view) records, or null (set up here)
    const ViewAux* aux;
};

template <Geo G, int R, int VB, int NG, int MinBlocks>
__global__ void __launch_bounds__(NG * kBpThreads, MinBlocks)
    bp_tile_tma_sk(const float* __restrict__ proj, float* __restrict__ img,
                   const double* __restrict__ t0, const double* __restrict__ t1,
                   const double* __restrict__ t2, const TileConst c, const SkConst k)
{
    constexpr int kTY = (kBpThreads / 32) * R;
    constexpr int kTilePix = kTileX * kTY;
    __shared__ int s_last;
    grid_dep_wait();  // launched as a dependent of the kernel before it
    const int ctas = static_cast<int>(gridDim.x);
    const long long U = k.units;
    const long long u0 = sk_unit_begin(blockIdx.x, ctas, U);
    const long long u1 = sk_unit_begin(blockIdx.x + 1, ctas, U);
    for (long long t = u0 / k.nb; t * k.nb < u1; ++t) {
        const long long tu = t * k.nb;
        const int b0 = static_cast<int>((u0 > tu ? u0 : tu) - tu);
        const int b1 = static_cast<int>((u1 < tu + k.nb ? u1 : tu + k.nb) - tu);
        const int item = static_cast<int>(t / k.tiles_per_item);
        const int tl = static_cast<int>(t % k.tiles_per_item);
        const int tx = tl % k.tiles_x, ty = tl / k.tiles_x;
        const int first = sk_cta_of(tu, ctas, U), last = sk_cta_of(tu + k.nb - 1, ctas, U);
        if (first == last) {  // the whole tile is this CTA's
            if (!tile_forward<G, R, VB, NG>(proj, img, t0, t1, t2, c, tx, ty, item, 0, -1, nullptr, k.rec, k.aux))
                return;
            continue;
        }
        float* seg = k.partial + (static_cast<size_t>(t) * k.maxseg + (blockIdx.x - first)) * kTilePix;
        if (!tile_forward<G, R, VB, NG>(proj, img, t0, t1, t2, c, tx, ty, item, b0, b1, seg, k.rec, k.aux)) return;
        __threadfence();  // this segment is visible before it is counted
        __syncthreads();
        if (threadIdx.x == 0) s_last = atomicAdd(k.counter + t, 1) == last - first;
        __syncthreads();
        if (s_last) {
            __threadfence();
            const float* base = k.partial + static_cast<size_t>(t) * k.maxseg * kTilePix;
            float* I = img + static_cast<size_t>(item) * c.img_stride;
            for (int idx = threadIdx.x; idx < kTilePix; idx += NG * kBpThreads) {
                const int ix = tx * kTileX + idx % kTileX, iy = ty * kTY + idx / kTileX;
                float v = __ldcg(base + idx);
                for (int sg = 1; sg <= last - first; ++sg) v += __ldcg(base + sg * kTilePix + idx);
                if (ix < c.nx && iy < c.ny) I[static_cast<size_t>(iy) * c.nx + ix] = v * c.scale;
            }
            if (threadIdx.x == 0) k.counter[t] = 0;  // zero again for the next launch
        }
    }
}

// ---- host: window bounds --------------------------------------------------

constexpr double kPi = 3.14159265358979323846;

// Bound on the channel span of one tile for any view (in channels).
int fan_window(int ns, double ds, double dso, double dsd, int nx, int ny, double dx, double dy,
               double ox, double oy, int tile_y = kTileY)
{
    const double hx = ((nx - 1) / 2.0 + std::fabs(ox)) * dx, hy = ((ny - 1) / 2.0 + std::fabs(oy)) * dy;
    const double rimg = std::sqrt(hx * hx + hy * hy);  // farthest pixel centre from the iso-centre
    const double rt = 0.5 * std::sqrt(std::pow(kTileX * dx, 2) + std::pow(tile_y * dy, 2));
    const double dmin = dso - rimg - rt;
    if (dmin <= rt * 1.05) return ns + 2;  // a tile may reach the source: stage whole rows
    const double span = 2.0 * std::asin(std::min(1.0, rt / dmin)) * dsd / ds;
    const int w = static_cast<int>(std::ceil(span)) + 8;
    return std::min(w, ns + 2);
}

int par_window(int ns, double ds, double dx, double dy, int tile_y = kTileY)
{
    const double span = std::sqrt(std::pow(kTileX * dx, 2) + std::pow(tile_y * dy, 2)) / ds;
    const int w = static_cast<int>(std::ceil(span)) + 8;
    return std::min(w, ns + 2);
}

// The window every single-geometry kernel uses for a geometry (forward,
// either staging, and the adjoint): the same window centre gives the same
// positions, so the adjoint transposes the forward exactly.
inline int tile_window(int w)
{
    return std::max(w, 32);
}

}  // namespace
}  // namespace ctr
