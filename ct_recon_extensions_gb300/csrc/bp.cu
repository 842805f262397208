// Pixel-driven backprojection (fan, fan with an angle list, parallel,
// parallel single-view) and the exact adjoints of fan and parallel BP.
//
// FP32 path (the fast path).  A CTA owns a kTileX x kTileY pixel tile; each
// thread owns kRowsPerThread pixels of one column and keeps their sums in
// registers across all views.  Views are processed in blocks of kViewBlock:
// for each view the CTA computes, from the tile corners, the window of
// detector channels the tile can project into (for a fan the angular extent
// of a convex tile seen from the source is reached at its corners; for a
// parallel beam the projection is affine), and stages that window into
// shared memory as (p[i], p[i+1]-p[i]) pairs, zero outside the detector.  A
// pixel-view update is then: channel position, floor/fraction, one 8-byte
// shared load and one FMA for the interpolation.  The window length W is a
// host-side bound over all tiles and views; a kernel that meets a wider
// window raises kFlagWindowOverflow and clamps (never reads out of bounds).
//
// Reference semantics kept exactly: the term of a view is included iff the
// channel position s satisfies 0 <= s <= ns-1 (src/bp_fan_2d.cc:71); the
// interpolation is between floor(s) and floor(s)+1; the fan weight is
// dsd^2/(d^2+r^2) with dsd^2 and the orbit factor applied once at the end.
//
// FP64 path: one thread per pixel with the reference's own arithmetic order,
// reading the caller's FP64 tables (src/bp_fan_2d.cc:46-91,
// src/bp_par_2d.cc:51-90, src/bp_par_2d_sv.cc:55-92).
//
// Adjoints: the FP32 adjoint reuses the tile/window structure and scatters
// each pixel's two taps into a shared-memory window accumulator; windows are
// then added to the sinogram with one global atomic per channel and view
// (the sinogram is zeroed first).  Summation order therefore varies between
// runs at the FP32 rounding level.  The FP64 adjoint uses global atomics per
// tap.
#include <cfloat>

#include "ctr_common.cuh"

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
    float poly[6];         // fan: atan polynomial scaled by dsd/ds
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

// Detector window [lo, lo+W) that covers every tap of the tile for one view;
// *interior is set when every pixel of the tile projects at least one channel
// inside the detector (no inclusion test needed) and the window fits.
template <Geo G>
__device__ int window_start(float2 vp, float x0, float x1, float y0, float y1, const TileConst& c,
                            bool* interior)
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
    if (full || !(smin == smin) || !(smax == smax)) return -1;
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
// has landed, the CTA rewrites it as (p[i], p[i+1]-p[i]) pairs, zero off the
// detector, so an interpolation is one 8-byte shared load and one FMA.
//
// Interior fast path (every tap of the tile on the detector): the floor and
// fraction of s come from adding 2^23 - 0.5 (round-to-nearest of s - 1/2 lands
// the integer part in the low mantissa bits; s in [1, 2^22)), and for the fan
// atan(r/d) is the minimax polynomial below when |r/d| <= kAtanTmax on the
// whole tile, with an approximate reciprocal of d.

// atan(t) ~= t*P(t^2), |t| <= 0.6, max relative error 3.28e-08 (Remez, degree 5
// in t^2; coefficients from gen_atan_poly.py).
constexpr double kAtanPoly[6] = {9.99999967214467378e-01, -3.33326573611355148e-01,
                                 1.99772013637297047e-01, -1.39992597733896912e-01,
                                 9.42086263445095634e-02, -4.04465160162714304e-02};
constexpr float kAtanTmax = 0.6f;
constexpr float kMagic = 8388608.0f;       // 2^23
constexpr float kMagicHalf = 8388607.5f;   // 2^23 - 1/2
constexpr unsigned kMagicBits = 0x4B000000u;
constexpr int kGroups = 2;
constexpr int kBlockViews = kGroups * kViewBlock;
constexpr int kTmaThreads = kGroups * kBpThreads;
constexpr int kModeEdge = 0, kModeFast = 2;

struct ViewP {
    float2 vp;
    int lo;     // first staged channel
    int mode;   // kModeEdge or kModeFast
    int gx;     // TMA coordinate of the slot (16-byte aligned)
    int shift;  // lo's offset inside the slot
};

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for an mbarrier phase for at most ~1 s; false on timeout.
__device__ bool mbar_wait_bounded(unsigned bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > 1000000000ull) return false;
    }
    return true;
}

// TMA bulk copy (no tensor map): `bytes` (multiple of 16) from a 16-byte aligned
// global address to a 16-byte aligned shared address, completing on `bar`.
__device__ __forceinline__ void bulk_load(unsigned dst, const void* src, unsigned bytes, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(reinterpret_cast<unsigned long long>(src)), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ float2 lds_f2(unsigned addr)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

// Channel position on the interior fast path (shared by the forward and the
// adjoint so that both take bit-identical taps).  Fan: xs = dso + x sin b,
// xc = x cos b; parallel: xs = x cos t / ds + cents.  Returns s; *w is the fan
// distance weight 1/(d^2+r^2).
template <Geo G>
__device__ __forceinline__ float fast_s(float xs, float xc, float y, float2 vp, const TileConst& c,
                                        float* w)
{
    if constexpr (G == Geo::kFan) {
        const float d = fmaf(-y, vp.y, xs);
        const float rr = fmaf(y, vp.x, xc);
        const float t = rr * rcp_approx(d);
        const float z = t * t;
        float p = fmaf(z, c.poly[5], c.poly[4]);
        p = fmaf(z, p, c.poly[3]);
        p = fmaf(z, p, c.poly[2]);
        p = fmaf(z, p, c.poly[1]);
        p = fmaf(z, p, c.poly[0]);
        *w = rcp_approx(fmaf(d, d, rr * rr));
        return fmaf(t, p, c.cents);
    } else {
        *w = 1.0f;
        return fmaf(y, vp.y, xs);
    }
}

template <Geo G>
__device__ __forceinline__ void fast_xs(float x, float2 vp, const TileConst& c, float* xs, float* xc)
{
    if constexpr (G == Geo::kFan) {
        *xs = fmaf(x, vp.x, c.dso);
        *xc = x * vp.y;
    } else {
        *xs = fmaf(x, vp.x, c.cents);
        *xc = 0.0f;
    }
}

// Per-view parameters, window and path for one tile (thread-local).
template <Geo G>
__device__ ViewP view_setup(const double* __restrict__ t2, int ia, int item, float x0, float x1,
                            float y0, float y1, const TileConst& c)
{
    ViewP P;
    P.vp = view_params<G>(t2, ia, c);
    bool inner;
    P.lo = window_start<G>(P.vp, x0, x1, y0, y1, c, &inner);
    bool fast = inner;
    if constexpr (G == Geo::kFan) {
        // polynomial atan needs d > 0 and |r/d| <= kAtanTmax on the whole tile
        // (r/d is a linear-fractional function: extremes at the corners)
        const float xs[2] = {x0, x1}, ys[2] = {y0, y1};
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const float d = fmaf(-ys[j], P.vp.y, fmaf(xs[i], P.vp.x, c.dso));
                const float r = fmaf(xs[i], P.vp.y, ys[j] * P.vp.x);
                fast = fast && d > 0.0f && fabsf(r) <= kAtanTmax * d;
            }
    }
    P.mode = fast ? kModeFast : kModeEdge;
    const long long start = (static_cast<long long>(item) * c.na + ia) * c.ns + P.lo;
    P.gx = static_cast<int>(start & ~3ll);
    P.shift = static_cast<int>(start - P.gx);
    return P;
}

template <Geo G>
__global__ void __launch_bounds__(kTmaThreads, 2)
    bp_tile_tma_f32(const float* __restrict__ proj, float* __restrict__ img,
                    const double* __restrict__ t0, const double* __restrict__ t1,
                    const double* __restrict__ t2, const TileConst c)
{
    // TMA destinations must be 128-byte aligned: align the dynamic region here
    // and give every view slot a 128-byte multiple stride (WS)
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    unsigned char* smem = smem_dyn + ((128u - (smem_u32(smem_dyn) & 127u)) & 127u);
    float* raw = reinterpret_cast<float*>(smem);  // [2][kBlockViews][WS]
    float2* pairs = reinterpret_cast<float2*>(smem + 2 * kBlockViews * c.WS * sizeof(float));
    __shared__ ViewP s_par[3][kBlockViews];
    __shared__ __align__(8) unsigned long long s_bar[2];
    __shared__ int s_ok;

    const int tid = threadIdx.x;
    const int group = tid / kBpThreads;
    const int lt = tid - group * kBpThreads;
    const int lane = lt & 31, warp = lt >> 5;
    const int tx0 = blockIdx.x * kTileX, ty0 = blockIdx.y * kTileY;
    const int item = blockIdx.z;
    const int nblocks = (c.na + kBlockViews - 1) / kBlockViews;

    auto px = [&](int ix) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t0[ix]);
        else return static_cast<float>((ix - c.centx) * c.dx);
    };
    auto py = [&](int iy) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t1[iy]);
        else return static_cast<float>((c.centy - iy) * c.dy);
    };
    const float cx0 = px(tx0), cx1 = px(min(tx0 + kTileX - 1, c.nx - 1));
    const float cy0 = py(ty0), cy1 = py(min(ty0 + kTileY - 1, c.ny - 1));

    auto setup_block = [&](int b) {
        if (b < nblocks && tid < kBlockViews) {
            const int ia = b * kBlockViews + tid;
            if (ia < c.na) s_par[b % 3][tid] = view_setup<G>(t2, ia, item, cx0, cx1, cy0, cy1, c);
        }
    };
    // one elected thread: arm the slot's barrier and issue the block's copies
    // Slot j of block b receives sinogram elements [gx, gx + WB) of the flattened
    // array (gx a multiple of 4, so the source is 16-byte aligned), clipped to
    // [0, total4) where total4 = total rounded down to 4 elements; the
    // conversion below reads the clipped-away elements from global directly.
    auto issue_block = [&](int b) {
        if (b >= nblocks) return;
        const int nv = min(kBlockViews, c.na - b * kBlockViews);
        const unsigned bar = smem_u32(&s_bar[b & 1]);
        unsigned bytes = 0;
        for (int j = 0; j < nv; ++j) {
            const long long g0 = max(static_cast<long long>(s_par[b % 3][j].gx), 0ll);
            const long long g1 = min(static_cast<long long>(s_par[b % 3][j].gx) + c.WB, c.total4);
            if (g1 > g0) bytes += static_cast<unsigned>((g1 - g0) * sizeof(float));
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bar, bytes);
        float* slot = raw + (b & 1) * kBlockViews * c.WS;
        for (int j = 0; j < nv; ++j) {
            const long long gx = s_par[b % 3][j].gx;
            const long long g0 = max(gx, 0ll), g1 = min(gx + c.WB, c.total4);
            if (g1 > g0)
                bulk_load(smem_u32(slot + j * c.WS + (g0 - gx)), proj + g0,
                          static_cast<unsigned>((g1 - g0) * sizeof(float)), bar);
        }
    };

    setup_block(0);
    setup_block(1);
    if (tid == 0) {
        // every copy destination must be 128-byte aligned; check before issuing any
        const bool aligned = (smem_u32(raw) & 127u) == 0 && (c.WS * sizeof(float)) % 128 == 0;
        s_ok = aligned;
        if (!aligned) raise_flag(kFlagMisaligned);
        mbar_init(smem_u32(&s_bar[0]), 1);
        mbar_init(smem_u32(&s_bar[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (!s_ok) return;
    if (tid == 0) {
        issue_block(0);
        issue_block(1);
    }

    const int ixc = min(tx0 + lane, c.nx - 1);
    const float x = px(ixc);
    float y[kRowsPerThread], acc[kRowsPerThread];
#pragma unroll
    for (int r = 0; r < kRowsPerThread; ++r) {
        y[r] = py(min(ty0 + warp * kRowsPerThread + r, c.ny - 1));
        acc[r] = 0.0f;
    }
    const unsigned pairs_u32 = smem_u32(pairs);

    for (int b = 0; b < nblocks; ++b) {
        setup_block(b + 2);
        if (tid == 0) s_ok = mbar_wait_bounded(smem_u32(&s_bar[b & 1]), (b >> 1) & 1);
        __syncthreads();
        if (!s_ok) {  // a copy never landed: report and leave (no copy of ours is pending)
            if (tid == 0) raise_flag(kFlagWaitTimeout);
            return;
        }
        const int nv = min(kBlockViews, c.na - b * kBlockViews);
        const float* slot = raw + (b & 1) * kBlockViews * c.WS;
        for (int idx = tid; idx < nv * c.W; idx += kTmaThreads) {
            const int j = idx / c.W, k = idx - j * c.W;
            const ViewP& P = s_par[b % 3][j];
            const int g = P.lo + k;  // channel of element k
            const long long gi = static_cast<long long>(P.gx) + P.shift + k;  // flat index
            const float* src = slot + j * c.WS + P.shift + k;
            auto at = [&](int gg, long long ii, const float* sp) -> float {
                if (gg < 0 || gg >= c.ns) return 0.0f;  // off the detector
                return ii < c.total4 ? *sp : __ldg(proj + ii);
            };
            const float p0 = at(g, gi, src);
            const float p1 = at(g + 1, gi + 1, src + 1);
            pairs[idx] = make_float2(p0, p1 - p0);
        }
        __syncthreads();
        if (tid == 0) issue_block(b + 2);  // its slot's raw data is consumed

        const int jb = group * kViewBlock;
        const int je = min(jb + kViewBlock, nv);
        for (int j = jb; j < je; ++j) {
            const ViewP P = s_par[b % 3][j];
            const int ia = b * kBlockViews + j;
            if (P.mode == kModeFast) {
                // index of s = bits(v) - kMagicBits, v = fl(s + 2^23 - 1/2)
                const unsigned base = pairs_u32 + 8u * static_cast<unsigned>(j * c.W) -
                                      8u * (kMagicBits + static_cast<unsigned>(P.lo));
                float xs, xc;
                fast_xs<G>(x, P.vp, c, &xs, &xc);
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r) {
                    float w;
                    const float s = fast_s<G>(xs, xc, y[r], P.vp, c, &w);
                    const float v = s + kMagicHalf;
                    const float u = s - (v - kMagic);
                    const float2 pv = lds_f2(base + 8u * __float_as_uint(v));
                    if constexpr (G == Geo::kFan) acc[r] = fmaf(fmaf(u, pv.y, pv.x), w, acc[r]);
                    else acc[r] = fmaf(u, pv.y, acc[r] + pv.x);
                }
            } else {
                const float2* wj = pairs + j * c.W;
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r) {
                    float w, u;
                    int k;
                    const float s = channel_of<G>(x, y[r], P.vp, c, &w);
                    const int iyc = min(ty0 + warp * kRowsPerThread + r, c.ny - 1);
                    if (edge_tap<G>(s, ixc, iyc, ia, P.lo, t0, t1, t2, c, &k, &u)) {
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
    // add the second group's sums to the first's, in that order
    float* red = reinterpret_cast<float*>(pairs);
    if (group == 1) {
#pragma unroll
        for (int r = 0; r < kRowsPerThread; ++r) red[r * kBpThreads + lt] = acc[r];
    }
    __syncthreads();
    if (group == 0) {
        float* I = img + static_cast<size_t>(item) * c.img_stride;
        const int ix = tx0 + lane;
#pragma unroll
        for (int r = 0; r < kRowsPerThread; ++r) {
            const int iy = ty0 + warp * kRowsPerThread + r;
            if (ix < c.nx && iy < c.ny)
                I[static_cast<size_t>(iy) * c.nx + ix] = (acc[r] + red[r * kBpThreads + lt]) * c.scale;
        }
    }
}

// Adjoint FP32 tile kernel: img [ny][nx] -> grad [na][ns] (grad pre-zeroed).
// Takes exactly the taps of the forward (same path choice per view and tile,
// same arithmetic) and scatters them into a shared-memory window per view,
// which is then added to the sinogram with one atomic per channel.
template <Geo G>
__global__ void __launch_bounds__(kBpThreads, 2)
    bp_tile_adj_f32(const float* __restrict__ img, float* __restrict__ grad,
                    const double* __restrict__ t0, const double* __restrict__ t1,
                    const double* __restrict__ t2, const TileConst c)
{
    extern __shared__ float accw[];  // [kViewBlock][W]
    __shared__ ViewP s_par[kViewBlock];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tx0 = blockIdx.x * kTileX, ty0 = blockIdx.y * kTileY;
    auto px = [&](int ix) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t0[ix]);
        else return static_cast<float>((ix - c.centx) * c.dx);
    };
    auto py = [&](int iy) -> float {
        if constexpr (G == Geo::kFan) return static_cast<float>(t1[iy]);
        else return static_cast<float>((c.centy - iy) * c.dy);
    };
    const int ix = tx0 + lane;
    const int ixc = min(ix, c.nx - 1);
    const float x = px(ixc);
    const float* I = img + blockIdx.z * c.img_stride;
    float y[kRowsPerThread], val[kRowsPerThread];
#pragma unroll
    for (int r = 0; r < kRowsPerThread; ++r) {
        const int iy = ty0 + warp * kRowsPerThread + r;
        y[r] = py(min(iy, c.ny - 1));
        val[r] = (ix < c.nx && iy < c.ny) ? I[static_cast<size_t>(iy) * c.nx + ix] * c.scale : 0.0f;
    }
    const float cx0 = px(tx0), cx1 = px(min(tx0 + kTileX - 1, c.nx - 1));
    const float cy0 = py(ty0), cy1 = py(min(ty0 + kTileY - 1, c.ny - 1));
    float* G_ = grad + blockIdx.z * c.proj_stride;

    for (int v0 = 0; v0 < c.na; v0 += kViewBlock) {
        const int nv = min(kViewBlock, c.na - v0);
        if (threadIdx.x < nv)
            s_par[threadIdx.x] = view_setup<G>(t2, v0 + threadIdx.x, blockIdx.z, cx0, cx1, cy0, cy1, c);
        for (int idx = threadIdx.x; idx < nv * c.W; idx += kBpThreads) accw[idx] = 0.0f;
        __syncthreads();
        for (int j = 0; j < nv; ++j) {
            const ViewP P = s_par[j];
            float* aj = accw + j * c.W;
            if (P.mode == kModeFast) {
                float xs, xc;
                fast_xs<G>(x, P.vp, c, &xs, &xc);
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r) {
                    float w;
                    const float s = fast_s<G>(xs, xc, y[r], P.vp, c, &w);
                    const float v = s + kMagicHalf;
                    const float u = s - (v - kMagic);
                    const int k = static_cast<int>(__float_as_uint(v) - kMagicBits) - P.lo;
                    const float t = val[r] * w;
                    if (t != 0.0f) {
                        atomicAdd(aj + k, t - t * u);
                        atomicAdd(aj + k + 1, t * u);
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r) {
                    if (val[r] == 0.0f) continue;
                    float w, u;
                    int k;
                    const float s = channel_of<G>(x, y[r], P.vp, c, &w);
                    const int iyc = min(ty0 + warp * kRowsPerThread + r, c.ny - 1);
                    if (edge_tap<G>(s, ixc, iyc, v0 + j, P.lo, t0, t1, t2, c, &k, &u)) {
                        const float t = val[r] * w;
                        atomicAdd(aj + k, t - t * u);
                        atomicAdd(aj + k + 1, t * u);
                    }
                }
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < nv * c.W; idx += kBpThreads) {
            const int j = idx / c.W, k = idx - j * c.W;
            const int g = s_par[j].lo + k;
            const float a = accw[idx];
            if (g >= 0 && g < c.ns && a != 0.0f)
                atomicAdd(G_ + static_cast<size_t>(v0 + j) * c.ns + g, a);
        }
        __syncthreads();
    }
}

// ---- FP64 kernels (reference arithmetic) -------------------------------------

template <bool kScaled>
__global__ void bp_fan_f64(const double* __restrict__ proj, double* __restrict__ img,
                           const double* __restrict__ xpos, const double* __restrict__ ypos,
                           const double* __restrict__ sincos, int ns, int na, int nx, int ny,
                           double dso, double dsd, double ds, double cents, double scale,
                           size_t proj_stride, size_t img_stride)
{
    const size_t n = static_cast<size_t>(nx) * ny;
    const size_t tid = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    const int ix = static_cast<int>(tid % nx), iy = static_cast<int>(tid / nx);
    const double* P = proj + blockIdx.y * proj_stride;
    const double x = xpos[ix], y = ypos[iy];
    double sum = 0.0;
    for (int ia = 0; ia < na; ++ia) {
        const double d = dso + x * sincos[2 * ia] - y * sincos[2 * ia + 1];
        const double r = x * sincos[2 * ia + 1] + y * sincos[2 * ia];
        const double s = atan2(r, d) * dsd / ds + cents;
        const double w = dsd * dsd / (d * d + r * r);
        if (s >= 0 && s <= ns - 1) {
            const int is1 = static_cast<int>(floor(s));
            const int is2 = static_cast<int>(ceil(s));
            const double u = s - is1;
            sum += ((1 - u) * P[is1 + static_cast<size_t>(ia) * ns] +
                    u * P[is2 + static_cast<size_t>(ia) * ns]) * w;
        }
    }
    img[blockIdx.y * img_stride + tid] = kScaled ? sum * scale : sum;
}

template <bool kScaled>
__global__ void bp_fan_adj_f64(const double* __restrict__ img, double* __restrict__ grad,
                               const double* __restrict__ xpos, const double* __restrict__ ypos,
                               const double* __restrict__ sincos, int ns, int na, int nx, int ny,
                               double dso, double dsd, double ds, double cents, double scale,
                               size_t proj_stride, size_t img_stride)
{
    const size_t n = static_cast<size_t>(nx) * ny;
    const size_t tid = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    const int ix = static_cast<int>(tid % nx), iy = static_cast<int>(tid / nx);
    double* Gr = grad + blockIdx.y * proj_stride;
    const double v = img[blockIdx.y * img_stride + tid] * (kScaled ? scale : 1.0);
    if (v == 0.0) return;
    const double x = xpos[ix], y = ypos[iy];
    for (int ia = 0; ia < na; ++ia) {
        const double d = dso + x * sincos[2 * ia] - y * sincos[2 * ia + 1];
        const double r = x * sincos[2 * ia + 1] + y * sincos[2 * ia];
        const double w = dsd * dsd / (d * d + r * r);
        const double s = atan2(r, d) * dsd / ds + cents;
        if (s >= 0 && s <= ns - 1) {
            const int is1 = static_cast<int>(floor(s));
            const int is2 = static_cast<int>(ceil(s));
            const double u = s - is1;
            atomicAdd(Gr + is1 + static_cast<size_t>(ia) * ns, v * (w * (1 - u)));
            atomicAdd(Gr + is2 + static_cast<size_t>(ia) * ns, v * (w * u));
        }
    }
}

__global__ void bp_par_f64(const double* __restrict__ proj, double* __restrict__ img,
                           const double* __restrict__ xcos, const double* __restrict__ ysin,
                           int ns, int na, int nx, int ny, double ds, double cents, double orbit,
                           size_t proj_stride, size_t img_stride)
{
    const size_t n = static_cast<size_t>(nx) * ny;
    const size_t tid = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    const int ix = static_cast<int>(tid % nx), iy = static_cast<int>(tid / nx);
    const double* P = proj + blockIdx.y * proj_stride;
    const double* xc = xcos + static_cast<size_t>(ix) * na;
    const double* ys = ysin + static_cast<size_t>(iy) * na;
    double sum = 0.0;
    for (int ia = 0; ia < na; ++ia) {
        const double s = (xc[ia] + ys[ia]) / ds + cents;
        if (s >= 0 && s <= ns - 1) {
            const int is1 = static_cast<int>(floor(s));
            const int is2 = static_cast<int>(ceil(s));
            const double u = s - is1;
            sum += (1 - u) * P[is1 + static_cast<size_t>(ia) * ns] +
                   u * P[is2 + static_cast<size_t>(ia) * ns];
        }
    }
    img[blockIdx.y * img_stride + tid] = sum * orbit;
}

__global__ void bp_par_adj_f64(const double* __restrict__ img, double* __restrict__ grad,
                               const double* __restrict__ xcos, const double* __restrict__ ysin,
                               int ns, int na, int nx, int ny, double ds, double cents,
                               double orbit, size_t proj_stride, size_t img_stride)
{
    const size_t n = static_cast<size_t>(nx) * ny;
    const size_t tid = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    const int ix = static_cast<int>(tid % nx), iy = static_cast<int>(tid / nx);
    double* Gr = grad + blockIdx.y * proj_stride;
    const double v = img[blockIdx.y * img_stride + tid] * orbit;
    if (v == 0.0) return;
    const double* xc = xcos + static_cast<size_t>(ix) * na;
    const double* ys = ysin + static_cast<size_t>(iy) * na;
    for (int ia = 0; ia < na; ++ia) {
        const double s = (xc[ia] + ys[ia]) / ds + cents;
        if (s >= 0 && s <= ns - 1) {
            const int is1 = static_cast<int>(floor(s));
            const int is2 = static_cast<int>(ceil(s));
            const double u = s - is1;
            atomicAdd(Gr + is1 + static_cast<size_t>(ia) * ns, (1 - u) * v);
            atomicAdd(Gr + is2 + static_cast<size_t>(ia) * ns, u * v);
        }
    }
}

// Single-view BP: a CTA owns kSvPix consecutive pixels of one row and all
// views; the caller's xcos/ysin rows for those pixels are staged once.  The
// output [ny][nx][na] is written view-fastest (coalesced).
constexpr int kSvThreads = 256;
constexpr int kSvPix = 4;

template <typename T>
__global__ void __launch_bounds__(kSvThreads)
    bp_par_sv(const T* __restrict__ proj, T* __restrict__ img, const double* __restrict__ xcos,
              const double* __restrict__ ysin, int ns, int na, int nx, int ny, double ds,
              double cents, size_t proj_stride, size_t img_stride)
{
    const int iy = blockIdx.y;
    const int ix0 = blockIdx.x * kSvPix;
    const T* P = proj + blockIdx.z * proj_stride;
    T* O = img + blockIdx.z * img_stride;
    const double* ys = ysin + static_cast<size_t>(iy) * na;
    const int npix = min(kSvPix, nx - ix0);
    for (int idx = threadIdx.x; idx < npix * na; idx += kSvThreads) {
        const int p = idx / na, ia = idx - p * na;
        const int ix = ix0 + p;
        const double* xc = xcos + static_cast<size_t>(ix) * na;
        T out;
        if constexpr (sizeof(T) == 8) {
            const double s = (xc[ia] + ys[ia]) / ds + cents;
            if (s >= 0 && s <= ns - 1) {
                const int is1 = static_cast<int>(floor(s));
                const int is2 = static_cast<int>(ceil(s));
                const double u = s - is1;
                out = (1 - u) * P[is1 + static_cast<size_t>(ia) * ns] +
                      u * P[is2 + static_cast<size_t>(ia) * ns];
            } else {
                out = 0;
            }
        } else {
            // inclusion decided on the FP64 channel position, as the reference;
            // the position is then rounded once to FP32
            const double sd = (xc[ia] + ys[ia]) / ds + cents;
            const float s = static_cast<float>(sd);
            if (sd >= 0 && sd <= ns - 1) {
                const float fs = floorf(s);
                const float u = s - fs;
                const int is1 = static_cast<int>(fs);
                const int is2 = min(is1 + 1, ns - 1);
                const float p0 = P[is1 + static_cast<size_t>(ia) * ns];
                const float p1 = P[is2 + static_cast<size_t>(ia) * ns];
                out = fmaf(u, p1 - p0, p0);
            } else {
                out = 0.0f;
            }
        }
        O[(static_cast<size_t>(iy) * nx + ix) * na + ia] = out;
    }
}

// ---- host side ---------------------------------------------------------------

constexpr double kPi = 3.14159265358979323846;

// Bound on the channel span of one tile for any view (in channels).
int fan_window(int ns, double ds, double dso, double dsd, int nx, int ny, double dx, double dy,
               double ox, double oy)
{
    const double hx = ((nx - 1) / 2.0 + std::fabs(ox)) * dx, hy = ((ny - 1) / 2.0 + std::fabs(oy)) * dy;
    const double rimg = std::sqrt(hx * hx + hy * hy);  // farthest pixel centre from the iso-centre
    const double rt = 0.5 * std::sqrt(std::pow(kTileX * dx, 2) + std::pow(kTileY * dy, 2));
    const double dmin = dso - rimg - rt;
    if (dmin <= rt * 1.05) return ns + 2;  // a tile may reach the source: stage whole rows
    const double span = 2.0 * std::asin(std::min(1.0, rt / dmin)) * dsd / ds;
    const int w = static_cast<int>(std::ceil(span)) + 8;
    return std::min(w, ns + 2);
}

int par_window(int ns, double ds, double dx, double dy)
{
    const double span = std::sqrt(std::pow(kTileX * dx, 2) + std::pow(kTileY * dy, 2)) / ds;
    const int w = static_cast<int>(std::ceil(span)) + 8;
    return std::min(w, ns + 2);
}

template <class K>
int launch_tile(K kern, int W, dim3 grid, cudaStream_t stream, const char* what,
                const void* a0, void* a1, const double* xpos, const double* ypos,
                const double* sincos, const TileConst& c, bool adjoint)
{
    const size_t smem = static_cast<size_t>(kViewBlock) * W * (adjoint ? sizeof(float) : sizeof(float2));
    if (smem > 160 * 1024) return fail(CTR_ERR_UNSUPPORTED, "%s: window of %d channels too wide", what, W);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    kern<<<grid, kBpThreads, smem, stream>>>(static_cast<const float*>(a0), static_cast<float*>(a1),
                                             xpos, ypos, sincos, c);
    return check_launch(what);
}


// Forward dispatch: the bulk-copy kernel when its window fits 256 elements and
// the sinogram is 16-byte aligned, the cooperative kernel otherwise.
template <Geo G>
int launch_forward(const float* proj, float* img, const double* t0, const double* t1,
                   const double* t2, TileConst c, int batch, cudaStream_t stream, const char* what)
{
    dim3 grid(div_up(c.nx, kTileX), div_up(c.ny, kTileY), batch);
    c.W = std::max(c.W, 16);
    c.WB = (c.W + 4 + 3) / 4 * 4;
    c.WS = (c.WB + 31) / 32 * 32;
    const unsigned long long total = static_cast<unsigned long long>(c.proj_stride) * batch;
    c.total4 = static_cast<long long>(total & ~3ull);
    if (c.WB <= 256 && reinterpret_cast<uintptr_t>(proj) % 16 == 0 && total < (1ull << 31)) {
        const size_t smem = 128 + 2 * kBlockViews * c.WS * sizeof(float) + kBlockViews * c.W * sizeof(float2);
        cudaError_t e = cudaFuncSetAttribute(bp_tile_tma_f32<G>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
        bp_tile_tma_f32<G><<<grid, kTmaThreads, smem, stream>>>(proj, img, t0, t1, t2, c);
        return check_launch(what);
    }
    return launch_tile(bp_tile_f32_coop<G>, c.W, grid, stream, what, proj, img, t0, t1, t2, c, false);
}

struct FanArgs {
    unsigned ns, na, nx, ny;
    double ds, offset_s, dx, dy, offset_x, offset_y, dso, dsd;
    double scale;  // output scale (orbit factor or 1)
};

int check_fan(const FanArgs& a, const void* in, const void* out, const double* xpos,
              const double* ypos, const double* sc, int batch)
{
    if (!in || !out || !xpos || !ypos || !sc) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (a.ns < 1 || a.na < 1 || a.nx < 1 || a.ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (!(a.ds != 0.0) || !(a.dsd != 0.0)) return fail(CTR_ERR_INVALID_ARG, "ds and dsd must be nonzero");
    if (batch > 65535) return fail(CTR_ERR_UNSUPPORTED, "batch > 65535");
    return CTR_OK;
}

TileConst fan_const(const FanArgs& a, double extra_scale)
{
    TileConst c{};
    c.ns = a.ns; c.na = a.na; c.nx = a.nx; c.ny = a.ny;
    c.W = fan_window(a.ns, a.ds, a.dso, a.dsd, a.nx, a.ny, a.dx, a.dy, a.offset_x, a.offset_y);
    c.cents = static_cast<float>((a.ns - 1) / 2.0 + a.offset_s);
    c.nsm1 = static_cast<float>(a.ns - 1);
    c.dso = static_cast<float>(a.dso);
    c.K = static_cast<float>(a.dsd / a.ds);
    c.scale = static_cast<float>(a.dsd * a.dsd * extra_scale);
    c.ds_d = a.ds;
    c.cents_d = (a.ns - 1) / 2.0 + a.offset_s;
    c.dso_d = a.dso;
    c.dsd_d = a.dsd;
    for (int k = 0; k < 6; ++k) c.poly[k] = static_cast<float>(kAtanPoly[k] * a.dsd / a.ds);
    c.proj_stride = static_cast<size_t>(a.ns) * a.na;
    c.img_stride = static_cast<size_t>(a.nx) * a.ny;
    return c;
}

template <typename T>
int fan_forward(const FanArgs& a, const T* proj, T* img, const double* xpos, const double* ypos,
                const double* sc, int batch, cudaStream_t stream, bool scaled)
{
    int st = check_fan(a, proj, img, xpos, ypos, sc, batch);
    if (st) return st;
    if constexpr (sizeof(T) == 4) {
        TileConst c = fan_const(a, scaled ? a.scale : 1.0);
        return launch_forward<Geo::kFan>(proj, img, xpos, ypos, sc, c, batch, stream, "bp_fan_2d");
    } else {
        const double cents = (a.ns - 1) / 2.0 + a.offset_s;
        dim3 grid(div_up(static_cast<size_t>(a.nx) * a.ny, 128), batch);
        if (scaled)
            bp_fan_f64<true><<<grid, 128, 0, stream>>>(proj, img, xpos, ypos, sc, a.ns, a.na, a.nx,
                                                      a.ny, a.dso, a.dsd, a.ds, cents, a.scale,
                                                      static_cast<size_t>(a.ns) * a.na,
                                                      static_cast<size_t>(a.nx) * a.ny);
        else
            bp_fan_f64<false><<<grid, 128, 0, stream>>>(proj, img, xpos, ypos, sc, a.ns, a.na, a.nx,
                                                       a.ny, a.dso, a.dsd, a.ds, cents, 1.0,
                                                       static_cast<size_t>(a.ns) * a.na,
                                                       static_cast<size_t>(a.nx) * a.ny);
        return check_launch("bp_fan_2d_f64");
    }
}

template <typename T>
int fan_adjoint(const FanArgs& a, const T* img, T* grad, const double* xpos, const double* ypos,
                const double* sc, int batch, cudaStream_t stream, bool scaled)
{
    int st = check_fan(a, img, grad, xpos, ypos, sc, batch);
    if (st) return st;
    cudaError_t e = cudaMemsetAsync(grad, 0, sizeof(T) * static_cast<size_t>(a.ns) * a.na * batch, stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "zero grad: %s", cudaGetErrorString(e));
    if constexpr (sizeof(T) == 4) {
        TileConst c = fan_const(a, scaled ? a.scale : 1.0);
        dim3 grid(div_up(a.nx, kTileX), div_up(a.ny, kTileY), batch);
        return launch_tile(bp_tile_adj_f32<Geo::kFan>, c.W, grid, stream, "bp_fan_2d_grad", img,
                           grad, xpos, ypos, sc, c, true);
    } else {
        const double cents = (a.ns - 1) / 2.0 + a.offset_s;
        dim3 grid(div_up(static_cast<size_t>(a.nx) * a.ny, 128), batch);
        if (scaled)
            bp_fan_adj_f64<true><<<grid, 128, 0, stream>>>(img, grad, xpos, ypos, sc, a.ns, a.na,
                                                          a.nx, a.ny, a.dso, a.dsd, a.ds, cents,
                                                          a.scale, static_cast<size_t>(a.ns) * a.na,
                                                          static_cast<size_t>(a.nx) * a.ny);
        else
            bp_fan_adj_f64<false><<<grid, 128, 0, stream>>>(img, grad, xpos, ypos, sc, a.ns, a.na,
                                                           a.nx, a.ny, a.dso, a.dsd, a.ds, cents,
                                                           1.0, static_cast<size_t>(a.ns) * a.na,
                                                           static_cast<size_t>(a.nx) * a.ny);
        return check_launch("bp_fan_2d_grad_f64");
    }
}

FanArgs fan_args(const ctr_fan_bp_param* p)
{
    FanArgs a{p->ns, p->na, p->nx, p->ny, p->ds, p->offset_s, p->dx, p->dy, p->offset_x,
              p->offset_y, p->dso, p->dsd, 1.0};
    // |orbit| / round(|na*orbit|/pi)  (reference src/bp_fan_2d.cc:59,87)
    const double factor = std::round(std::fabs(p->na * p->orbit) / kPi);
    a.scale = std::fabs(p->orbit) / factor;
    return a;
}

FanArgs angle_args(const ctr_fan_bp_angle_param* p)
{
    return FanArgs{p->ns, p->na, p->nx, p->ny, p->ds, p->offset_s, p->dx, p->dy, p->offset_x,
                   p->offset_y, p->dso, p->dsd, 1.0};
}

int check_par(const ctr_par_param* p, const void* in, const void* out, const double* xcos,
              const double* ysin, int batch)
{
    if (!p || !in || !out || !xcos || !ysin) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (p->ns < 1 || p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (!(p->ds != 0.0)) return fail(CTR_ERR_INVALID_ARG, "ds must be nonzero");
    if (batch > 65535) return fail(CTR_ERR_UNSUPPORTED, "batch > 65535");
    return CTR_OK;
}

TileConst par_const(const ctr_par_param* p)
{
    TileConst c{};
    c.ns = p->ns; c.na = p->na; c.nx = p->nx; c.ny = p->ny;
    c.W = par_window(p->ns, p->ds, p->dx, p->dy);
    c.cents = static_cast<float>((p->ns - 1) / 2.0 + p->offset_s);
    c.nsm1 = static_cast<float>(p->ns - 1);
    c.scale = static_cast<float>(p->orbit);
    c.orbit_start = p->orbit_start;
    c.orbit = p->orbit;
    c.inv_ds = 1.0 / p->ds;
    c.centx = (p->nx - 1) / 2.0 + p->offset_x;
    c.centy = (p->ny - 1) / 2.0 + p->offset_y;
    c.dx = p->dx;
    c.dy = p->dy;
    c.ds_d = p->ds;
    c.cents_d = (p->ns - 1) / 2.0 + p->offset_s;
    c.proj_stride = static_cast<size_t>(p->ns) * p->na;
    c.img_stride = static_cast<size_t>(p->nx) * p->ny;
    return c;
}

template <typename T>
int par_forward(const ctr_par_param* p, const T* proj, T* img, const double* xcos,
                const double* ysin, int batch, cudaStream_t stream)
{
    int st = check_par(p, proj, img, xcos, ysin, batch);
    if (st) return st;
    if constexpr (sizeof(T) == 4) {
        TileConst c = par_const(p);
        return launch_forward<Geo::kPar>(proj, img, xcos, ysin, nullptr, c, batch, stream, "bp_par_2d");
    } else {
        const double cents = (p->ns - 1) / 2.0 + p->offset_s;
        dim3 grid(div_up(static_cast<size_t>(p->nx) * p->ny, 128), batch);
        bp_par_f64<<<grid, 128, 0, stream>>>(proj, img, xcos, ysin, p->ns, p->na, p->nx, p->ny,
                                             p->ds, cents, p->orbit,
                                             static_cast<size_t>(p->ns) * p->na,
                                             static_cast<size_t>(p->nx) * p->ny);
        return check_launch("bp_par_2d_f64");
    }
}

template <typename T>
int par_adjoint(const ctr_par_param* p, const T* img, T* grad, const double* xcos,
                const double* ysin, int batch, cudaStream_t stream)
{
    int st = check_par(p, img, grad, xcos, ysin, batch);
    if (st) return st;
    cudaError_t e = cudaMemsetAsync(grad, 0, sizeof(T) * static_cast<size_t>(p->ns) * p->na * batch, stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "zero grad: %s", cudaGetErrorString(e));
    if constexpr (sizeof(T) == 4) {
        TileConst c = par_const(p);
        dim3 grid(div_up(p->nx, kTileX), div_up(p->ny, kTileY), batch);
        return launch_tile(bp_tile_adj_f32<Geo::kPar>, c.W, grid, stream, "bp_par_2d_grad", img,
                           grad, xcos, ysin, nullptr, c, true);
    } else {
        const double cents = (p->ns - 1) / 2.0 + p->offset_s;
        dim3 grid(div_up(static_cast<size_t>(p->nx) * p->ny, 128), batch);
        bp_par_adj_f64<<<grid, 128, 0, stream>>>(img, grad, xcos, ysin, p->ns, p->na, p->nx,
                                                 p->ny, p->ds, cents, p->orbit,
                                                 static_cast<size_t>(p->ns) * p->na,
                                                 static_cast<size_t>(p->nx) * p->ny);
        return check_launch("bp_par_2d_grad_f64");
    }
}

template <typename T>
int par_single_view(const ctr_par_param* p, const T* proj, T* img, const double* xcos,
                    const double* ysin, int batch, cudaStream_t stream)
{
    int st = check_par(p, proj, img, xcos, ysin, batch);
    if (st) return st;
    const double cents = (p->ns - 1) / 2.0 + p->offset_s;
    dim3 grid(div_up(p->nx, kSvPix), p->ny, batch);
    bp_par_sv<T><<<grid, kSvThreads, 0, stream>>>(proj, img, xcos, ysin, p->ns, p->na, p->nx,
                                                  p->ny, p->ds, cents,
                                                  static_cast<size_t>(p->ns) * p->na,
                                                  static_cast<size_t>(p->nx) * p->ny * p->na);
    return check_launch("bp_par_2d_sv");
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_bp_fan_2d_f32(const ctr_fan_bp_param* p, const float* proj, float* img,
                      const double* xpos, const double* ypos, const double* sincostbl,
                      int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_forward<float>(fan_args(p), proj, img, xpos, ypos, sincostbl, batch, stream, true);
}
int ctr_bp_fan_2d_f64(const ctr_fan_bp_param* p, const double* proj, double* img,
                      const double* xpos, const double* ypos, const double* sincostbl,
                      int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_forward<double>(fan_args(p), proj, img, xpos, ypos, sincostbl, batch, stream, true);
}
int ctr_bp_fan_2d_grad_f32(const ctr_fan_bp_param* p, const float* img, float* grad,
                           const double* xpos, const double* ypos, const double* sincostbl,
                           int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_adjoint<float>(fan_args(p), img, grad, xpos, ypos, sincostbl, batch, stream, true);
}
int ctr_bp_fan_2d_grad_f64(const ctr_fan_bp_param* p, const double* img, double* grad,
                           const double* xpos, const double* ypos, const double* sincostbl,
                           int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_adjoint<double>(fan_args(p), img, grad, xpos, ypos, sincostbl, batch, stream, true);
}

int ctr_bp_fan_2d_angle_f32(const ctr_fan_bp_angle_param* p, const float* proj, float* img,
                            const double* xpos, const double* ypos, const double* sincostbl,
                            int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_forward<float>(angle_args(p), proj, img, xpos, ypos, sincostbl, batch, stream, false);
}
int ctr_bp_fan_2d_angle_f64(const ctr_fan_bp_angle_param* p, const double* proj, double* img,
                            const double* xpos, const double* ypos, const double* sincostbl,
                            int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_forward<double>(angle_args(p), proj, img, xpos, ypos, sincostbl, batch, stream, false);
}
int ctr_bp_fan_2d_angle_grad_f32(const ctr_fan_bp_angle_param* p, const float* img,
                                 float* grad, const double* xpos, const double* ypos,
                                 const double* sincostbl, int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_adjoint<float>(angle_args(p), img, grad, xpos, ypos, sincostbl, batch, stream, false);
}
int ctr_bp_fan_2d_angle_grad_f64(const ctr_fan_bp_angle_param* p, const double* img,
                                 double* grad, const double* xpos, const double* ypos,
                                 const double* sincostbl, int batch, cudaStream_t stream)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null param");
    return fan_adjoint<double>(angle_args(p), img, grad, xpos, ypos, sincostbl, batch, stream, false);
}

int ctr_bp_par_2d_f32(const ctr_par_param* p, const float* proj, float* img,
                      const double* xcos, const double* ysin, const int* buffer, int batch,
                      cudaStream_t stream)
{
    (void)buffer;
    return par_forward<float>(p, proj, img, xcos, ysin, batch, stream);
}
int ctr_bp_par_2d_f64(const ctr_par_param* p, const double* proj, double* img,
                      const double* xcos, const double* ysin, const int* buffer, int batch,
                      cudaStream_t stream)
{
    (void)buffer;
    return par_forward<double>(p, proj, img, xcos, ysin, batch, stream);
}
int ctr_bp_par_2d_grad_f32(const ctr_par_param* p, const float* img, float* grad,
                           const double* xcos, const double* ysin, int batch,
                           cudaStream_t stream)
{
    return par_adjoint<float>(p, img, grad, xcos, ysin, batch, stream);
}
int ctr_bp_par_2d_grad_f64(const ctr_par_param* p, const double* img, double* grad,
                           const double* xcos, const double* ysin, int batch,
                           cudaStream_t stream)
{
    return par_adjoint<double>(p, img, grad, xcos, ysin, batch, stream);
}
int ctr_bp_par_2d_sv_f32(const ctr_par_param* p, const float* proj, float* img,
                         const double* xcos, const double* ysin, const int* buffer, int batch,
                         cudaStream_t stream)
{
    (void)buffer;
    return par_single_view<float>(p, proj, img, xcos, ysin, batch, stream);
}
int ctr_bp_par_2d_sv_f64(const ctr_par_param* p, const double* proj, double* img,
                         const double* xcos, const double* ysin, const int* buffer, int batch,
                         cudaStream_t stream)
{
    (void)buffer;
    return par_single_view<double>(p, proj, img, xcos, ysin, batch, stream);
}

}  // extern "C"
