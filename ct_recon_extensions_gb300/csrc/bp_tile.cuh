// Device side of the FP32 pixel-driven backprojectors, shared by the
// single-geometry entry points (bp.cu) and the batched plan (batch.cu): view
// parameters, detector windows, the fast interior and exact edge tap paths,
// and the tile bodies.  Everything here has internal linkage per file.
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
constexpr int kRowsPerThread = 4;
constexpr int kTileY = (kBpThreads / 32) * kRowsPerThread;
constexpr int kViewBlock = 16;

enum class Geo { kFan, kPar };

// Per-launch constants of the FP32 tile kernels.
struct TileConst {
    int ns, na, nx, ny;
    int W;                 // staged window length (channels)
    float cents;           // (ns-1)/2 + offset_s
    float nsm1;            // ns - 1
    float dso, K;          // fan: source distance, dsd/ds
    float scale;           // applied once to the final sum
    double orbit_start, orbit;  // parallel: view angle = orbit_start + ia*orbit
    double inv_ds;         // parallel: 1/ds
    double centx, centy, dx, dy;  // parallel pixel grid
    double ds_d, cents_d, dso_d, dsd_d;  // FP64 geometry for the exact edge test
    float poly[4][6];      // fan: the atan polynomial variants, scaled by dsd/ds
    int WB;                // TMA box (elements) per view: >= W + 4, multiple of 4
    int WS;                // shared slot stride per view: WB rounded up to 128 bytes
    long long total4;      // sinogram elements of the launch, rounded down to 4
    size_t proj_stride, img_stride;
};

// FP32 channel positions are within ~3e-4 channels of the reference's FP64
// value (s up to ~2e3, plus atan2f error).  Within kEdgeEps of a detector end
// the inclusion decision is recomputed in FP64 from the caller's tables.
constexpr float kEdgeEps = 2e-3f;

// ---- per-view parameters ---------------------------------------------------
// Fan: (sin b, cos b) from the caller's table.  Parallel: (cos t / ds,
// sin t / ds) from the geometry, with t = orbit_start + ia*orbit.
template <Geo G>
__device__ __forceinline__ float2 view_params(const double* __restrict__ sincos, int ia,
                                              const TileConst& c)
{
    if constexpr (G == Geo::kFan) {
        return make_float2(static_cast<float>(sincos[2 * ia]), static_cast<float>(sincos[2 * ia + 1]));
    } else {
        double sa, ca;
        ::sincos(c.orbit_start + ia * c.orbit, &sa, &ca);
        return make_float2(static_cast<float>(ca * c.inv_ds), static_cast<float>(sa * c.inv_ds));
    }
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Channel position of pixel (x, y) for a view, and the fan distance weight
// 1/(d^2 + r^2) (dsd^2 is applied with the final scale).
template <Geo G>
__device__ __forceinline__ float channel_of(float x, float y, float2 vp, const TileConst& c,
                                            float* w)
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

// One pixel-view tap on an edge view: inclusion decided as the reference does
// (exactly, in FP64, near the detector ends); returns false when excluded.
template <Geo G>
__device__ __forceinline__ bool edge_tap(float s, int ix, int iy, int ia, int lo,
                                         const double* t0, const double* t1, const double* t2,
                                         const TileConst& c, int* k, float* u)
{
    float fs;
    if (fabsf(s) < kEdgeEps || fabsf(s - c.nsm1) < kEdgeEps) {
        const double sd = channel_exact<G>(ix, iy, ia, t0, t1, t2, c);
        if (!(sd >= 0.0 && sd <= static_cast<double>(c.ns - 1))) return false;
        const double fd = floor(sd);
        fs = static_cast<float>(fd);
        *u = static_cast<float>(sd - fd);
    } else {
        if (!(s >= 0.0f && s <= c.nsm1)) return false;
        fs = floorf(s);
        *u = s - fs;
    }
    *k = min(max(static_cast<int>(fs) - lo, 0), c.W - 2);
    return true;
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
__device__ int window_start(float2 vp, float x0, float x1, float y0, float y1, const TileConst& c,
                            bool* interior, bool* off = nullptr)
{
    float smin = FLT_MAX, smax = -FLT_MAX;
    bool full = false;
    const float xs[2] = {x0, x1}, ys[2] = {y0, y1};
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if constexpr (G == Geo::kFan) {
                const float d = fmaf(-ys[j], vp.y, fmaf(xs[i], vp.x, c.dso));
                if (d <= 0.0f) full = true;
            }
            float w;
            const float s = channel_of<G>(xs[i], ys[j], vp, c, &w);
            smin = fminf(smin, s);
            smax = fmaxf(smax, s);
        }
    }
    *interior = false;
    if (off) *off = false;
    if (full || !(smin == smin) || !(smax == smax)) return -1;
    if (off) *off = smax < -kSkipEps || smin > c.nsm1 + kSkipEps;
    int lo = static_cast<int>(floorf(smin)) - 2;
    int hi = static_cast<int>(floorf(smax)) + 3;
    const bool fits = hi - lo + 1 <= c.W;
    *interior = fits && smin >= 1.0f && smax <= c.nsm1 - 1.0f;
    lo = max(lo, -1);
    hi = min(hi, c.ns);
    if (hi - lo + 1 > c.W && lo <= c.ns && hi >= -1) raise_flag(kFlagWindowOverflow);
    return min(lo, c.ns);
}

// Forward FP32 tile kernel with cooperative (plain-load) staging: proj [na][ns]
// -> img [ny][nx] (batch in grid.z).  t0/t1/t2: fan xpos/ypos/sincostbl,
// parallel xcos/ysin/unused.  Used where the TMA kernel below does not apply
// (windows wider than one 256-element box, unaligned buffers).
template <Geo G>
__global__ void __launch_bounds__(kBpThreads, 2)
    bp_tile_f32_coop(const float* __restrict__ proj, float* __restrict__ img,
                const double* __restrict__ t0, const double* __restrict__ t1,
                const double* __restrict__ t2, const TileConst c)
{
    extern __shared__ float2 win[];  // [kViewBlock][W]
    __shared__ float2 s_vp[kViewBlock];
    __shared__ int s_lo[kViewBlock];
    __shared__ int s_in[kViewBlock];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tx0 = blockIdx.x * kTileX, ty0 = blockIdx.y * kTileY;
    const float* P = proj + blockIdx.z * c.proj_stride;

    auto px = [&](int ix) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t0[ix]);
        else return static_cast<float>((ix - c.centx) * c.dx);
    };
    auto py = [&](int iy) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t1[iy]);
        else return static_cast<float>((c.centy - iy) * c.dy);
    };
    const int ixc = min(tx0 + lane, c.nx - 1);
    const float x = px(ixc);
    float y[kRowsPerThread], acc[kRowsPerThread];
#pragma unroll
    for (int r = 0; r < kRowsPerThread; ++r) {
        y[r] = py(min(ty0 + warp * kRowsPerThread + r, c.ny - 1));
        acc[r] = 0.0f;
    }
    const float cx0 = px(tx0), cx1 = px(min(tx0 + kTileX - 1, c.nx - 1));
    const float cy0 = py(ty0), cy1 = py(min(ty0 + kTileY - 1, c.ny - 1));

    for (int v0 = 0; v0 < c.na; v0 += kViewBlock) {
        const int nv = min(kViewBlock, c.na - v0);
        if (threadIdx.x < nv) {
            const float2 vp = view_params<G>(t2, v0 + threadIdx.x, c);
            bool inner;
            s_vp[threadIdx.x] = vp;
            s_lo[threadIdx.x] = window_start<G>(vp, cx0, cx1, cy0, cy1, c, &inner);
            s_in[threadIdx.x] = inner;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < nv * c.W; idx += kBpThreads) {
            const int j = idx / c.W, k = idx - j * c.W;
            const int g = s_lo[j] + k;
            const float* row = P + static_cast<size_t>(v0 + j) * c.ns;
            const float p0 = (g >= 0 && g < c.ns) ? __ldg(row + g) : 0.0f;
            const float p1 = (g + 1 >= 0 && g + 1 < c.ns) ? __ldg(row + g + 1) : 0.0f;
            win[idx] = make_float2(p0, p1 - p0);
        }
        __syncthreads();
        for (int j = 0; j < nv; ++j) {
            const float2 vp = s_vp[j];
            const int lo = s_lo[j];
            const float2* wj = win + j * c.W;
            if (s_in[j]) {
                // every tap of the tile is on the detector and inside the window
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r) {
                    float w;
                    const float s = channel_of<G>(x, y[r], vp, c, &w);
                    const float fs = floorf(s);
                    const float2 pv = wj[static_cast<int>(fs) - lo];
                    const float v = fmaf(s - fs, pv.y, pv.x);
                    if constexpr (G == Geo::kFan) acc[r] = fmaf(v, w, acc[r]);
                    else acc[r] += v;
                }
            } else {
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r) {
                    float w, u;
                    int k;
                    const float s = channel_of<G>(x, y[r], vp, c, &w);
                    const int iyc = min(ty0 + warp * kRowsPerThread + r, c.ny - 1);
                    if (edge_tap<G>(s, ixc, iyc, v0 + j, lo, t0, t1, t2, c, &k, &u)) {
                        const float2 pv = wj[k];
                        const float v = fmaf(u, pv.y, pv.x);
                        if constexpr (G == Geo::kFan) acc[r] = fmaf(v, w, acc[r]);
                        else acc[r] += v;
                    }
                }
            }
        }
        __syncthreads();
    }
    float* I = img + blockIdx.z * c.img_stride;
    const int ix = tx0 + lane;
#pragma unroll
    for (int r = 0; r < kRowsPerThread; ++r) {
        const int iy = ty0 + warp * kRowsPerThread + r;
        if (ix < c.nx && iy < c.ny) I[static_cast<size_t>(iy) * c.nx + ix] = acc[r] * c.scale;
    }
}

// ---- TMA-fed forward kernel ---------------------------------------------------
//
// Same tile as bp_tile_f32_coop, but a CTA runs two view groups of 256 threads
// on the same 32x32 tile (each group takes half of every block of
// 2*kViewBlock views; the two partial sums are added in a fixed order at the
// end), and the detector windows reach shared memory through the TMA engine:
// one cp.async.bulk copy per view (16-byte aligned start in the flattened
// sinogram, a 128-byte aligned shared slot), issued two view blocks ahead
// into double-buffered raw slots, each block completed on its own mbarrier
// (waits are bounded and report kFlagWaitTimeout).  Once a slot
// has landed, the CTA rewrites it as (q[k], d[k]) pairs, d[k] = p[k+1] - p[k]
// and q[k] = p[k] - k d[k] (k the channel less the window start lo), zero off
// the detector, so an interpolation at s' = s - lo in [k, k+1] is one 8-byte
// shared load and one FMA, q[k] + s' d[k], with no fraction of s'.
//
// Interior fast path (every tap of the tile on the detector): s' comes out of
// the position's last FMA with cents - lo in place of cents, its floor from
// adding 2^23 - 0.5 (round-to-nearest of s' - 1/2 lands the integer part in
// the low mantissa bits; s' in [1, 2^22)), and for the fan
// atan(r/d) is one of the minimax polynomials below (the lowest degree whose
// range covers |r/d| on the whole tile, up to 0.6), with an approximate
// reciprocal of d.

// atan(t) ~= t*P(t^2), minimax for relative error (Remez; gen_atan_poly.py),
// four variants of about the same error: a tile takes the lowest degree whose
// range covers all its pixels.  |t| <= 0.6: degree 5 in t^2, max relative error
// 3.28e-08; |t| <= 0.45: degree 4, 3.87e-08; |t| <= 0.3: degree 3, 4.84e-08;
// |t| <= 0.15: degree 2, 4.93e-08.
constexpr int kAtanVariants = 4;
__host__ __device__ constexpr float atan_tmax(int v)
{
    return v == 0 ? 0.6f : v == 1 ? 0.45f : v == 2 ? 0.3f : 0.15f;
}
constexpr double kAtanPoly[kAtanVariants][6] = {
    {9.99999967214467378e-01, -3.33326573611355148e-01, 1.99772013637297047e-01, -1.39992597733896912e-01,
     9.42086263445095634e-02, -4.04465160162714304e-02},
    {9.99999961331696996e-01, -3.33323584754777580e-01, 1.99603534902473234e-01, -1.37111734158844867e-01,
     7.55531535813081662e-02, 0.0},
    {9.99999951640157425e-01, -3.33315939607756684e-01, 1.99016376594526256e-01, -1.24757817537760357e-01,
     0.0, 0.0},
    {9.99999950700421469e-01, -3.33293746601247498e-01, 1.95275580886984462e-01, 0.0, 0.0, 0.0}};
constexpr float kMagic = 8388608.0f;       // 2^23
constexpr float kMagicHalf = 8388607.5f;   // 2^23 - 1/2
constexpr unsigned kMagicBits = 0x4B000000u;
constexpr int kGroups = 2;
constexpr int kBlockViews = kGroups * kViewBlock;
constexpr int kTmaThreads = kGroups * kBpThreads;
constexpr int kModeEdge = 0, kModeSkip = 1, kModeFast = 2;
// A fast view's mode: a multiple of 8 (kModeFastBase, or the forward tile's
// shared slot base) plus the atan variant in the low two bits.
constexpr int kModeFastBase = 8;

struct ViewP {
    float2 vp;
    int lo;     // first staged channel
    int mode;   // kModeEdge, kModeSkip, or >= kModeFast: the interior fast path
                // (the forward tile stores the view's shared slot base there)
};
// Parallel beam: also the channel position of the tile's first pixel less lo,
// from FP64, so that fast-path positions add only in-tile offsets in FP32.
struct ViewPar : ViewP {
    float cen;
    int pad;
};
template <Geo G> struct ViewSel { using type = ViewP; };
template <> struct ViewSel<Geo::kPar> { using type = ViewPar; };
template <Geo G> using ViewT = typename ViewSel<G>::type;
constexpr size_t kViewBytesMax = sizeof(ViewPar);

// Fast-path origin of positions less the window start: the detector centre
// (fan) or the tile's first pixel (parallel).
template <Geo G>
__device__ __forceinline__ float view_cen(const ViewT<G>& P, const TileConst& c)
{
    if constexpr (G == Geo::kFan) return c.cents - static_cast<float>(P.lo);
    else return P.cen;
}

__device__ __forceinline__ bool mode_fast(int m) { return static_cast<unsigned>(m) >= kModeFast; }

__device__ __forceinline__ float2 lds_f2(unsigned addr)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

// Channel position on the interior fast path (shared by the forward and the
// adjoint), relative to the tile's window start lo, from ViewP.cen.  Fan (x, y
// absolute): xs = dso + x sin b, xc = x cos b, s - lo = K atan(r/d) + cen;
// parallel (x, y offsets from the tile's first pixel): xs = x cos t / ds + cen,
// s - lo = xs + y sin t / ds.  Returns s - lo (below the window length); *w is
// the fan distance weight 1/(d^2+r^2).
// V = the atan variant (fan; 0 for the parallel beam).
template <Geo G, int V = 0>
__device__ __forceinline__ float fast_s(float xs, float xc, float y, float2 vp, float cen,
                                        const TileConst& c, float* w)
{
    if constexpr (G == Geo::kFan) {
        constexpr int deg = 5 - V;
        const float d = fmaf(-y, vp.y, xs);
        const float rr = fmaf(y, vp.x, xc);
        const float t = rr * rcp_approx(d);
        const float z = t * t;
        float p = c.poly[V][deg];
#pragma unroll
        for (int k = deg - 1; k >= 0; --k) p = fmaf(z, p, c.poly[V][k]);
        *w = rcp_approx(fmaf(d, d, rr * rr));
        return fmaf(t, p, cen);
    } else {
        *w = 1.0f;
        return fmaf(y, vp.y, xs);
    }
}

template <Geo G>
__device__ __forceinline__ void fast_xs(float x, float2 vp, float cen, const TileConst& c, float* xs,
                                        float* xc)
{
    if constexpr (G == Geo::kFan) {
        *xs = fmaf(x, vp.x, c.dso);
        *xc = x * vp.y;
    } else {
        *xs = fmaf(x, vp.x, cen);
        *xc = 0.0f;
    }
}

// Per-view parameters, window and path for one tile (thread-local).
template <Geo G>
__device__ ViewT<G> view_setup(const double* __restrict__ t0, const double* __restrict__ t1,
                               const double* __restrict__ t2, int ia, int ix0, int iy0, float x0,
                               float x1, float y0, float y1, const TileConst& c)
{
    ViewT<G> P;
    if constexpr (G == Geo::kFan) {
        P.vp = view_params<G>(t2, ia, c);
    } else {
        // FP32 slopes: on the fast path they multiply offsets within the tile
        // only (the tile's origin comes from the FP64 tables below)
        float sf, cf;
        sincosf(static_cast<float>(c.orbit_start + ia * c.orbit), &sf, &cf);
        const float ids = static_cast<float>(c.inv_ds);
        P.vp = make_float2(cf * ids, sf * ids);
    }
    bool inner, off;
    P.lo = window_start<G>(P.vp, x0, x1, y0, y1, c, &inner, &off);
    bool fast = inner;
    if constexpr (G == Geo::kFan) {
        // polynomial atan needs d > 0 and |r/d| <= atan_tmax(0) on the whole
        // tile (r/d is a linear-fractional function: extremes at the corners);
        // the tile takes the lowest-degree variant that covers it
        const float xs[2] = {x0, x1}, ys[2] = {y0, y1};
        float tmax = 0.0f;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const float d = fmaf(-ys[j], P.vp.y, fmaf(xs[i], P.vp.x, c.dso));
                const float r = fmaf(xs[i], P.vp.y, ys[j] * P.vp.x);
                fast = fast && d > 0.0f && fabsf(r) <= atan_tmax(0) * d;
                tmax = fmaxf(tmax, fabsf(r) / d);
            }
        int v = 0;
#pragma unroll
        for (int k = 1; k < kAtanVariants; ++k)
            if (tmax <= atan_tmax(k)) v = k;
        P.mode = fast ? kModeFastBase + v : (off ? kModeSkip : kModeEdge);
    } else {
        P.mode = fast ? kModeFastBase : (off ? kModeSkip : kModeEdge);
    }
    if constexpr (G == Geo::kPar) {
        // s(x0, y0) - lo in FP64 from the caller's x cos t / y sin t tables
        // (src/bp_par_2d.cc:70), (ix0, iy0) the tile's first pixel: the fast
        // path adds only offsets within the tile in FP32 (at most a tile's
        // extent in channels)
        P.cen = static_cast<float>((t0[static_cast<size_t>(ix0) * c.na + ia] +
                                    t1[static_cast<size_t>(iy0) * c.na + ia]) * c.inv_ds +
                                   c.cents_d - P.lo);
        P.pad = 0;
    }
    return P;
}

// Pixel coordinates on the fast path: absolute for the fan, offsets from the
// tile's first pixel (x0, y0) for the parallel beam (exact: both are on the
// pixel grid).
template <Geo G>
__device__ __forceinline__ float fast_coord(float v, float v0)
{
    if constexpr (G == Geo::kFan) return v;
    else return v - v0;
}

// The fast-path taps of one view for a thread's R pixels (atan variant V).
template <Geo G, int V, int R>
__device__ __forceinline__ void fast_rows(float xs, float xc, const float (&yf)[R], float2 vp, float cen,
                                          const TileConst& c, unsigned base, float (&part)[R])
{
#pragma unroll
    for (int r = 0; r < R; ++r) {
        float w;
        const float s = fast_s<G, V>(xs, xc, yf[r], vp, cen, c, &w);
        const float2 pv = lds_f2(base + 8u * __float_as_uint(s + kMagicHalf));
        if constexpr (G == Geo::kFan) part[r] = fmaf(fmaf(s, pv.y, pv.x), w, part[r]);
        else part[r] += fmaf(s, pv.y, pv.x);
    }
}

// One tile (tile_x, tile_y) of item `item`, over its view blocks
// [b_begin, b_end) (b_end < 0: all); all 512 threads of the CTA call it.
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
                                             int b_end = -1, float* __restrict__ partial = nullptr)
{
    constexpr int kTY = (kBpThreads / 32) * R;  // tile height
    constexpr int kBV = NG * VB;                // views per staged block
    constexpr int kThreads = NG * kBpThreads;   // NG view groups of 256 threads
    // Dynamic shared memory, 128-byte aligned here: raw slots [2][kBV][WS]
    // (every slot stride a 128-byte multiple), pairs [2][kBV][W], then one
    // view record (ViewT<G>) per view of the whole scan.
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    unsigned char* smem = smem_dyn + ((128u - (smem_u32(smem_dyn) & 127u)) & 127u);
    float* raw = reinterpret_cast<float*>(smem);
    float2* pairs = reinterpret_cast<float2*>(smem + 2 * kBV * c.WS * sizeof(float));
    ViewT<G>* views = reinterpret_cast<ViewT<G>*>(pairs + 2 * kBV * c.W);
    __shared__ __align__(8) unsigned long long s_bar[2];
    __shared__ int s_ok;

    const int tid = threadIdx.x;
    const int group = tid / kBpThreads;
    const int lt = tid - group * kBpThreads;
    const int lane = lt & 31, warp = lt >> 5;
    const int tx0 = tile_x * kTileX, ty0 = tile_y * kTY;
    const int nblocks = b_end < 0 ? (c.na + kBV - 1) / kBV : b_end;
    // double-buffer slots and barrier phases count from b_begin

    auto px = [&](int ix) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t0[ix]);
        else return static_cast<float>((ix - c.centx) * c.dx);
    };
    auto py = [&](int iy) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t1[iy]);
        else return static_cast<float>((c.centy - iy) * c.dy);
    };
    const float cx0 = px(tx0), cx1 = px(min(tx0 + kTileX - 1, c.nx - 1));
    const float cy0 = py(ty0), cy1 = py(min(ty0 + kTY - 1, c.ny - 1));

    // Slot j of block b receives sinogram elements [gx, gx + WB) of the flattened
    // array (gx = window start rounded down to 4 elements, so the source is
    // 16-byte aligned), clipped to [0, total4) where total4 = total rounded down
    // to 4 elements; the conversion below reads the clipped-away elements from
    // global directly.
    auto slot_start = [&](int ia) -> long long {
        return (static_cast<long long>(item) * c.na + ia) * c.ns + views[ia].lo;
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

    // per-view parameters, windows and paths of this tile for the whole scan;
    // a fast view keeps, in place of its mode, the shared address of its pair
    // slot minus 8 * kMagicBits (a multiple of 8), so a tap's address is that
    // plus 8 * bits(s' + 2^23 - 1/2), s' = s - lo; the low two bits keep the
    // atan variant (values below kModeFastBase fall back to the edge path)
    const unsigned pairs_base = smem_u32(pairs);
    const int ia_end = min(nblocks * kBV, c.na);
    for (int ia = b_begin * kBV + tid; ia < ia_end; ia += kThreads) {
        ViewT<G> P = view_setup<G>(t0, t1, t2, ia, tx0, ty0, cx0, cx1, cy0, cy1, c);
        if (mode_fast(P.mode)) {
            const int slot = ((ia / kBV - b_begin) & 1) * kBV + ia % kBV;
            const unsigned base = pairs_base + 8u * static_cast<unsigned>(slot * c.W) - 8u * kMagicBits;
            P.mode = base >= static_cast<unsigned>(kModeFastBase) ? static_cast<int>(base | (P.mode & 3))
                                                                 : kModeEdge;
        }
        views[ia] = P;
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

    const int ixc = min(tx0 + lane, c.nx - 1);
    const float x = px(ixc);
    const float xf = fast_coord<G>(x, cx0);
    float y[R], yf[R], acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        y[r] = py(min(ty0 + warp * R + r, c.ny - 1));
        yf[r] = fast_coord<G>(y[r], cy0);
        acc[r] = 0.0f;
    }

    const int wid = tid >> 5;  // warp of the CTA (0..15)
    for (int b = b_begin; b < nblocks; ++b) {
        const int lb = b - b_begin;
        // every thread waits for block b's copies (bounded); a timeout is
        // reported and the block proceeds, so no thread is left at a barrier
        if (!mbar_wait_bounded(smem_u32(&s_bar[lb & 1]), (lb >> 1) & 1) && tid == 0)
            raise_flag(kFlagWaitTimeout);
        const int nv = min(kBV, c.na - b * kBV);
        const float* slot = raw + (lb & 1) * kBV * c.WS;
        float2* pb = pairs + (lb & 1) * kBV * c.W;
        // one warp per view: rewrite the raw window as (p[k] - k d[k], d[k]) pairs,
        // d[k] = p[k+1] - p[k], k the channel less lo (a tap at s' = s - lo in
        // [k, k+1] is then one FMA: p[k] + (s' - k) d[k] = q[k] + s' d[k])
        for (int j = wid; j < nv; j += kThreads / 32) {
            const long long st = slot_start(b * kBV + j);
            const int lo = views[b * kBV + j].lo;
            const float* src = slot + j * c.WS + static_cast<int>(st & 3ll);
            float2* dst = pb + j * c.W;
            if (lo >= 0 && lo + c.W < c.ns && st + c.W < c.total4) {
                for (int k = lane; k < c.W; k += 32) {
                    const float p0 = src[k], d = src[k + 1] - p0;
                    dst[k] = make_float2(fmaf(-static_cast<float>(k), d, p0), d);
                }
            } else {  // a detector end or the array's ragged tail is in the window
                for (int k = lane; k < c.W; k += 32) {
                    auto at = [&](int gg, long long ii, const float* sp) -> float {
                        if (gg < 0 || gg >= c.ns) return 0.0f;  // off the detector
                        return ii < c.total4 ? *sp : __ldg(proj + ii);
                    };
                    const float p0 = at(lo + k, st + k, src + k);
                    const float d = at(lo + k + 1, st + k + 1, src + k + 1) - p0;
                    dst[k] = make_float2(fmaf(-static_cast<float>(k), d, p0), d);
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
        for (int j = jb; j < je; ++j) {
            const int ia = b * kBV + j;
            const ViewT<G> P = views[ia];
            if (mode_fast(P.mode)) {
                // floor of s' = bits(fl(s' + 2^23 - 1/2)) - kMagicBits
                const unsigned base = static_cast<unsigned>(P.mode) & ~3u;
                const float cen = view_cen<G>(P, c);
                float xs, xc;
                fast_xs<G>(xf, P.vp, cen, c, &xs, &xc);
                if constexpr (G == Geo::kFan) {
                    switch (P.mode & 3) {
                        case 0: fast_rows<G, 0, R>(xs, xc, yf, P.vp, cen, c, base, part); break;
                        case 1: fast_rows<G, 1, R>(xs, xc, yf, P.vp, cen, c, base, part); break;
                        case 2: fast_rows<G, 2, R>(xs, xc, yf, P.vp, cen, c, base, part); break;
                        default: fast_rows<G, 3, R>(xs, xc, yf, P.vp, cen, c, base, part); break;
                    }
                } else {
                    fast_rows<G, 0, R>(xs, xc, yf, P.vp, cen, c, base, part);
                }
            } else if (P.mode == kModeEdge) {
                const float2* wj = pb + j * c.W;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    float w, u;
                    int k;
                    const float s = channel_of<G>(x, y[r], P.vp, c, &w);
                    const int iyc = min(ty0 + warp * R + r, c.ny - 1);
                    if (edge_tap<G>(s, ixc, iyc, ia, P.lo, t0, t1, t2, c, &k, &u)) {
                        const float2 pv = wj[k];
                        const float v = fmaf(u, pv.y, fmaf(static_cast<float>(k), pv.y, pv.x));
                        if constexpr (G == Geo::kFan) part[r] = fmaf(v, w, part[r]);
                        else part[r] += v;
                    }
                }
            }
        }
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
            const int ix = tx0 + lane;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int iy = ty0 + warp * R + r;
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
                    const double* __restrict__ t2, const TileConst c)
{
    tile_forward<G, R, VB, NG>(proj, img, t0, t1, t2, c, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---- stream-K split of small launches ----------------------------------------
//
// A launch with few tiles (a 512^2 image is 128 tiles of 32 x 64) leaves SMs
// idle when each CTA owns whole tiles.  Here the work is cut into units of
// (tile, block of 2*VB views), tiles outer, and CTA c of G takes the
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
    int* counter;          // [tiles], zero at launch
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
            if (!tile_forward<G, R, VB, NG>(proj, img, t0, t1, t2, c, tx, ty, item)) return;
            continue;
        }
        float* seg = k.partial + (static_cast<size_t>(t) * k.maxseg + (blockIdx.x - first)) * kTilePix;
        if (!tile_forward<G, R, VB, NG>(proj, img, t0, t1, t2, c, tx, ty, item, b0, b1, seg)) return;
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

}  // namespace
}  // namespace ctr
