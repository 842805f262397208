// Pixel-driven backprojection (fan, fan with an angle list, parallel,
// parallel single-view) and the exact adjoints of fan and parallel BP.
//
// FP32 path (the fast path).  A CTA owns a kTileX x kTileY pixel tile; each
// thread owns kRowsPerThread pixels of one column and keeps their sums in
// registers across all views.  Views are processed in blocks: for each view
// the CTA computes, from the tile corners, the window of detector channels
// the tile can project into (for a fan the angular extent of a convex tile
// seen from the source is reached at its corners; for a parallel beam the
// projection is affine), and stages that window into shared memory as pairs,
// zero outside the detector.  A pixel-view update is then: the channel
// position relative to the window centre (tile-relative arithmetic,
// bp_tile.cuh), its rounding, one 8-byte shared load and one FMA for the
// interpolation.  The window length W is a host-side bound over all tiles and
// views; a kernel that meets a wider window raises kFlagWindowOverflow and
// clamps (never reads out of bounds).
//
// Reference semantics kept exactly: the term of a view is included iff the
// channel position s satisfies 0 <= s <= ns-1 (src/bp_fan_2d.cc:71); the
// interpolation is between floor(s) and floor(s)+1; the fan weight is
// dsd^2/(d^2+r^2) with dsd^2 and the orbit factor applied once at the end.
//
// FP64 path: one thread per pixel with the reference's own arithmetic order,
// reading the caller's FP64 tables (src/bp_fan_2d.cc:46-91,
// src/bp_par_2d.cc:51-90, src/bp_par_2d_sv.cc:55-92).  The FP64 adjoint uses
// global atomics per tap.
#include <cfloat>
#include <memory>
#include <type_traits>

#include "bp_tile.cuh"

namespace ctr {
namespace {

// ---- FP32 adjoint ---------------------------------------------------------------
//
// img [ny][nx] -> grad [na][ns] (grad pre-zeroed): the exact transpose of the
// FP32 forward.  It uses the forward's tiles (32 x kTileY), window, view
// records and position arithmetic (bp_tile.cuh), so every (pixel, view) gets
// the forward's channel index, fraction and weight.
//
// Work is split stream-K over (tile, block of kViewBlock views) units like the
// forward; no segment needs combining, because every CTA adds into the
// sinogram.  Per block, the CTA scatters each pixel's two taps into a window
// of 32-bit fixed-point accumulators per view in shared memory
// (red.shared.add.u32: integer shared atomics run at load speed without
// conflicts, float ones measured 3x slower), then adds each nonzero window
// entry to the sinogram with one global float atomic (so the summation order
// over tiles varies between runs at the FP32 rounding level).
//
// Fixed point: a tile's values are scaled by a power of two so that the
// largest |value| is below 2^fx_bits (fx_bits <= 20, chosen on the host so a
// window entry's sum of taps stays below 2^31); a tap t*u is rounded to an
// integer with one FMA (adding 1.5*2^23), and the two taps of a pixel add up
// to round(t) exactly.  The quantisation step is 2^-fx_bits of the tile's
// largest value.  Tiles holding non-finite values add every tap to the
// sinogram directly in FP32, as do fan tiles on the absolute path.
//
// Thread mapping per view: lanes along x (as the forward) where the position
// changes faster along x, along y otherwise; 32 neighbouring lanes then hit
// distinct or at most pairwise-equal accumulators.
struct AdjUnits {
    long long units;  // tiles x nb
    int nb;           // view blocks per tile
    int tiles_x, tiles_per_item;
    const FastRec* rec;  // a plan's per-(tile, view) records, or null (set up here)
    const ViewAux* aux;
};

constexpr int kAdjChunkBlocks = 64;  // view records set up per chunk of blocks

// A fast view's mode in the adjoint: the address of its accumulator slot plus
// 4 kc, less 4 kMagicBits, with the variant in the low bits.
__device__ __forceinline__ int adj_fast_mode(unsigned slot_addr, const TileConst& c, int mode)
{
    const unsigned base = slot_addr + 4u * static_cast<unsigned>(c.kc) - 4u * kMagicBits;
    const int v = mode_variant(mode);
    return base >= static_cast<unsigned>(kModeFastBase) ? static_cast<int>(base | static_cast<unsigned>(v))
                                                        : kModeEdgeRel + v;
}

// round(x) for |x| < 2^22 as an integer, by one FP32 add.
__device__ __forceinline__ int round_int(float x)
{
    return static_cast<int>(__float_as_uint(__fadd_rn(x, kMagic)) - kMagicBits);
}

// The two taps of two parallel-beam pixels whose fixed-point values tq are
// integers, tb = bits(tq + 1.5*2^23) (formed once per tile), at window-relative
// positions sig (j = round(sig) + kc, accumulator address base + 4 bits(sig +
// 1.5*2^23)): q1 = round(tq u) at j + 1 and tq - q1 at j, u = sig - round(sig)
// + 1/2 with the half folded into the rounding constant of the FMA.  The FP32
// steps of the two pixels run as packed pairs.
__device__ __forceinline__ void adj_taps_int2(unsigned base, float2 sig, float2 tq, unsigned tb0, unsigned tb1)
{
    const float2 vb = __fadd2_rn(sig, dup2(kMagic));
    const float2 d = sub2(sig, __fadd2_rn(vb, dup2(-kMagic)));
    const float2 q = __ffma2_rn(tq, d, __ffma2_rn(tq, dup2(0.5f), dup2(kMagic)));
    const unsigned a0 = base + 4u * __float_as_uint(vb.x), a1 = base + 4u * __float_as_uint(vb.y);
    const unsigned q0 = __float_as_uint(q.x), q1 = __float_as_uint(q.y);
    red_shared_u32(a0, tb0 - q0);
    red_shared_u32(a0 + 4u, q0 - kMagicBits);
    red_shared_u32(a1, tb1 - q1);
    red_shared_u32(a1 + 4u, q1 - kMagicBits);
}

// The two taps of two pixels with fixed-point values t at window-relative
// positions sig: (round(t) - q1) at j = round(sig) + kc and q1 = round(t u) at
// j + 1, u = sig - round(sig) + 1/2.  The FP32 steps run as packed pairs.
__device__ __forceinline__ void adj_taps2(unsigned base, float2 sig, float2 t)
{
    const float2 vb = __fadd2_rn(sig, dup2(kMagic));  // round(sig) in its bits: the address
    const float2 r = __fadd2_rn(vb, dup2(-kMagic));
    const float2 u = __fadd2_rn(sub2(sig, r), dup2(0.5f));
    const float2 q = __ffma2_rn(t, u, dup2(kMagic));
    const float2 tr = __fadd2_rn(t, dup2(kMagic));
    const unsigned a0 = base + 4u * __float_as_uint(vb.x), a1 = base + 4u * __float_as_uint(vb.y);
    const int q1a = static_cast<int>(__float_as_uint(q.x) - kMagicBits);
    const int q1b = static_cast<int>(__float_as_uint(q.y) - kMagicBits);
    const int q0a = static_cast<int>(__float_as_uint(tr.x) - kMagicBits) - q1a;
    const int q0b = static_cast<int>(__float_as_uint(tr.y) - kMagicBits) - q1b;
    red_shared_u32(a0, static_cast<unsigned>(q0a));
    red_shared_u32(a0 + 4u, static_cast<unsigned>(q1a));
    red_shared_u32(a1, static_cast<unsigned>(q0b));
    red_shared_u32(a1 + 4u, static_cast<unsigned>(q1b));
}

// Whether a view walks the tile x-major (its channel changes faster along x).
__device__ __forceinline__ bool adj_xmaj(const FastRec& P, const TileConst& c)
{
    return fabsf(P.p0) * c.dxf >= fabsf(P.p1) * c.dyf;
}

// 1 when every one of the n (<= 32) views at vr is x-major, 0 when every one
// is y-major, else -1 (warp-uniform).
__device__ __forceinline__ int block_major(const FastRec* vr, int n, const TileConst& c)
{
    const int lane = threadIdx.x & 31;
    const bool m = lane < n ? adj_xmaj(load_fast(vr + lane), c) : true;
    const bool yes = lane < n ? !m : true;
    return __all_sync(0xffffffffu, m) ? 1 : (__all_sync(0xffffffffu, yes) ? 0 : -1);
}

// The fast-path taps of one view for a thread's pixels, parallel beam: the
// x-major mapping (column oxx, rows oyx) or the y-major one (columns oxy[r &
// 3], rows oyy[r >> 2]); pixel pairs (r, r+1) packed.
template <int R>
__device__ __forceinline__ void adj_par_view(const FastRec& P, unsigned base, bool xmaj, float oxx,
                                             const float (&oyx)[R], const float (&oxy)[4],
                                             const float (&oyy)[R / 4], const float (&vx)[R],
                                             const float (&vy)[R], const unsigned (&tbx)[R],
                                             const unsigned (&tby)[R])
{
    const float2 p1 = dup2(P.p1);
    if (xmaj) {
        const float2 xs = dup2(par_xpart(oxx, P));
#pragma unroll
        for (int r = 0; r < R; r += 2)
            adj_taps_int2(base, __ffma2_rn(make_float2(oyx[r], oyx[r + 1]), p1, xs), make_float2(vx[r], vx[r + 1]),
                          tbx[r], tbx[r + 1]);
    } else {
        const float2 p0 = dup2(P.p0), cen = dup2(P.cen);
        const float2 xs01 = __ffma2_rn(make_float2(oxy[0], oxy[1]), p0, cen);
        const float2 xs23 = __ffma2_rn(make_float2(oxy[2], oxy[3]), p0, cen);
#pragma unroll
        for (int r = 0; r < R; r += 2)
            adj_taps_int2(base, __ffma2_rn(dup2(oyy[r >> 2]), p1, (r & 3) ? xs23 : xs01),
                          make_float2(vy[r], vy[r + 1]), tby[r], tby[r + 1]);
    }
}

// The same for the fan beam (variant V), pixel pairs packed.
template <int V, int R>
__device__ __forceinline__ void adj_fan_view(const FastRec& P, unsigned base, bool xmaj, float oxx,
                                             const float (&oyx)[R], const float (&oxy)[4],
                                             const float (&oyy)[R / 4], const float (&vx)[R],
                                             const float (&vy)[R], const TileConst& c)
{
    if (xmaj) {
        const FanX X = fan_xpart(oxx, P);
        const float2 xn = dup2(X.n), xd = dup2(X.d);
#pragma unroll
        for (int r = 0; r < R; r += 2) {
            float2 w;
            const float2 sig = fan_sigma2<V>(xn, xd, make_float2(oyx[r], oyx[r + 1]), P, c, &w);
            adj_taps2(base, sig, __fmul2_rn(make_float2(vx[r], vx[r + 1]), w));
        }
    } else {
        FanX X[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) X[q] = fan_xpart(oxy[q], P);
#pragma unroll
        for (int r = 0; r < R; r += 2) {
            const int q = r & 3;
            float2 w;
            const float2 sig = fan_sigma2<V>(make_float2(X[q].n, X[q + 1].n), make_float2(X[q].d, X[q + 1].d),
                                             dup2(oyy[r >> 2]), P, c, &w);
            adj_taps2(base, sig, __fmul2_rn(make_float2(vy[r], vy[r + 1]), w));
        }
    }
}

template <Geo G>
__global__ void __launch_bounds__(kBpThreads, 2)
    bp_tile_adj(const float* __restrict__ img, float* __restrict__ grad, const double* __restrict__ t0,
                const double* __restrict__ t1, const double* __restrict__ t2, const TileConst c,
                const AdjUnits k)
{
    constexpr int R = kRowsPerThread;
    extern __shared__ __align__(16) unsigned char adj_smem[];
    unsigned* win = reinterpret_cast<unsigned*>(adj_smem);  // [kViewBlock][W]
    FastRec* views = reinterpret_cast<FastRec*>(adj_smem + (kViewBlock * c.W * 4 + 15) / 16 * 16);
    ViewAux* vaux = reinterpret_cast<ViewAux*>(views + kAdjChunkBlocks * kViewBlock);
    __shared__ unsigned s_max[kBpThreads / 32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ctas = static_cast<int>(gridDim.x);
    const long long U = k.units;
    const long long u0 = sk_unit_begin(blockIdx.x, ctas, U);
    const long long u1 = sk_unit_begin(blockIdx.x + 1, ctas, U);
    const unsigned win_base = smem_u32(win);
    for (int i = tid; i < kViewBlock * c.W; i += kBpThreads) win[i] = 0u;  // the flush re-zeroes

    for (long long t = u0 / k.nb; t * k.nb < u1; ++t) {
        const long long tu = t * k.nb;
        const int b0 = static_cast<int>((u0 > tu ? u0 : tu) - tu);
        const int b1 = static_cast<int>((u1 < tu + k.nb ? u1 : tu + k.nb) - tu);
        const int item = static_cast<int>(t / k.tiles_per_item);
        const int tl = static_cast<int>(t % k.tiles_per_item);
        const TileBox B = tile_box<G>(t0, t1, tl % k.tiles_x, tl / k.tiles_x, kTileY, c);
        __syncthreads();  // s_max of the previous tile has been read by every warp
        const float* I = img + static_cast<size_t>(item) * c.img_stride;
        float* Gs = grad + static_cast<size_t>(item) * c.proj_stride;

        // pixels of the two mappings: x-major (column lane, rows warp*R + r) and
        // y-major (column warp*4 + (r & 3), row lane + 32 (r >> 2))
        float vx[R], vy[R], oyx[R], oxy[4], oyy[R / 4];
        const int ixx = min(B.tx0 + lane, c.nx - 1);
        const float oxx = off_x<G>(t0, ixx, B.ixm, c);
        unsigned m = 0u;
        bool bad = false;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int ix = B.tx0 + lane, iy = B.ty0 + warp * R + r;
            vx[r] = (ix < c.nx && iy < c.ny) ? I[static_cast<size_t>(iy) * c.nx + ix] : 0.0f;
            oyx[r] = off_y<G>(t1, min(iy, c.ny - 1), B.iym, c);
            const int jx = B.tx0 + warp * 4 + (r & 3), jy = B.ty0 + lane + 32 * (r >> 2);
            vy[r] = (jx < c.nx && jy < c.ny) ? I[static_cast<size_t>(jy) * c.nx + jx] : 0.0f;
            m = max(m, __float_as_uint(fabsf(vx[r])));
            bad = bad || !isfinite(vx[r]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) oxy[q] = off_x<G>(t0, min(B.tx0 + warp * 4 + q, c.nx - 1), B.ixm, c);
#pragma unroll
        for (int h = 0; h < R / 4; ++h) oyy[h] = off_y<G>(t1, min(B.ty0 + lane + 32 * h, c.ny - 1), B.iym, c);
        m = __reduce_max_sync(0xffffffffu, m);
        if (lane == 0) s_max[warp] = m;
        const bool any_bad = __syncthreads_or(bad) != 0;
        m = 0u;
#pragma unroll
        for (int w = 0; w < kBpThreads / 32; ++w) m = max(m, s_max[w]);
        if (m == 0u && !any_bad) continue;  // an all-zero tile adds nothing (uniform)
        int ex = 0;
        frexpf(__uint_as_float(m), &ex);
        const int sh = c.fx_bits - ex;  // values * 2^sh are below 2^fx_bits
        // per pixel: the scaled value; the parallel beam rounds it to an
        // integer once (its taps do not depend on the view) and keeps the
        // rounding's bit pattern
        unsigned tbx[R], tby[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            vx[r] = any_bad ? vx[r] * c.scale : ldexpf(vx[r], sh);
            vy[r] = any_bad ? vy[r] * c.scale : ldexpf(vy[r], sh);
            tbx[r] = __float_as_uint(__fadd_rn(vx[r], kMagic));
            tby[r] = __float_as_uint(__fadd_rn(vy[r], kMagic));
            if (G == Geo::kPar && !any_bad) {
                vx[r] = __fadd_rn(__uint_as_float(tbx[r]), -kMagic);
                vy[r] = __fadd_rn(__uint_as_float(tby[r]), -kMagic);
            }
        }
        const float back = ldexpf(c.scale, -sh);  // fixed point -> sinogram units

        for (int b = b0; b < b1; ++b) {
            if ((b - b0) % kAdjChunkBlocks == 0) {
                // view records of the next chunk of blocks (slot j of block b: win + j*W)
                const int va = b * kViewBlock;
                const int vb = min(min(b1, b + kAdjChunkBlocks) * kViewBlock, c.na);
                __syncthreads();
                for (int ia = va + tid; ia < vb; ia += kBpThreads) {
                    ViewRec P;
                    if (k.rec) {
                        const size_t ti = static_cast<size_t>(tl) * c.na + ia;
                        const FastRec F = k.rec[ti];
                        const ViewAux A = k.aux[ti];
                        P.p0 = F.p0;
                        P.p1 = F.p1;
                        P.cen = F.cen;
                        P.mode = F.mode;
                        P.e = A.e;
                        P.lo = A.lo;
                    } else {
                        P = view_setup<G>(t0, t1, t2, ia, B, c);
                    }
                    if (mode_fast(P.mode))
                        P.mode = adj_fast_mode(win_base + 4u * static_cast<unsigned>((ia % kViewBlock) * c.W), c,
                                               P.mode);
                    store_view(views, vaux, ia - va, P);
                }
                __syncthreads();
            }
            const int v0 = b * kViewBlock;
            const int nv = min(kViewBlock, c.na - v0);
            const FastRec* vb = views + (b - b0) % kAdjChunkBlocks * kViewBlock;
            const ViewAux* vab = vaux + (b - b0) % kAdjChunkBlocks * kViewBlock;
            // every view of the block on the fast path (one variant): no per-view dispatch
            const int fv = any_bad ? -1 : block_variant(vb, nv);
            if (fv >= 0) {
                // views of one walk direction (the usual case): no per-view test
                const int bm = block_major(vb, nv, c);
                if constexpr (G == Geo::kPar) {
                    auto par_block = [&](auto mc) {
                        constexpr int M = decltype(mc)::value;
                        auto one = [&](const FastRec& P) {
                            adj_par_view<R>(P, static_cast<unsigned>(P.mode) & ~3u, M < 0 ? adj_xmaj(P, c) : M == 1,
                                            oxx, oyx, oxy, oyy, vx, vy, tbx, tby);
                        };
                        int j = 0;
                        for (; j + 2 <= nv; j += 2) {  // two views per trip
                            const FastRec P0 = load_fast(vb + j), P1 = load_fast(vb + j + 1);
                            one(P0);
                            one(P1);
                        }
                        if (j < nv) one(load_fast(vb + j));
                    };
                    if (bm == 1) par_block(std::integral_constant<int, 1>{});
                    else if (bm == 0) par_block(std::integral_constant<int, 0>{});
                    else par_block(std::integral_constant<int, -1>{});
                } else {
                    auto fan_block = [&](auto vc) {
                        constexpr int V = decltype(vc)::value;
                        auto run = [&](auto mc) {
                            constexpr int M = decltype(mc)::value;
                            auto one = [&](const FastRec& P) {
                                adj_fan_view<V, R>(P, static_cast<unsigned>(P.mode) & ~3u,
                                                   M < 0 ? adj_xmaj(P, c) : M == 1, oxx, oyx, oxy, oyy, vx, vy, c);
                            };
                            int j = 0;
                            for (; j + 2 <= nv; j += 2) {  // two views per trip
                                const FastRec P0 = load_fast(vb + j), P1 = load_fast(vb + j + 1);
                                one(P0);
                                one(P1);
                            }
                            if (j < nv) one(load_fast(vb + j));
                        };
                        if (bm == 1) run(std::integral_constant<int, 1>{});
                        else if (bm == 0) run(std::integral_constant<int, 0>{});
                        else run(std::integral_constant<int, -1>{});
                    };
                    switch (fv) {
                        case 0: fan_block(std::integral_constant<int, 0>{}); break;
                        case 1: fan_block(std::integral_constant<int, 1>{}); break;
                        default: fan_block(std::integral_constant<int, 2>{}); break;
                    }
                }
            }
            for (int j = 0; j < (fv >= 0 ? 0 : nv); ++j) {
                const FastRec F = load_fast(vb + j);
                if (F.mode == kModeSkip) continue;
                const int ia = v0 + j;
                const unsigned slot = win_base + 4u * static_cast<unsigned>(j * c.W);
                const bool xmaj = adj_xmaj(F, c);
                if (mode_fast(F.mode) && !any_bad) {
                    const FastRec& P = F;
                    const unsigned base = static_cast<unsigned>(P.mode) & ~3u;
                    if constexpr (G == Geo::kPar) {
                        adj_par_view<R>(P, base, xmaj, oxx, oyx, oxy, oyy, vx, vy, tbx, tby);
                    } else {
                        switch (mode_variant(P.mode)) {
                            case 0: adj_fan_view<0, R>(P, base, xmaj, oxx, oyx, oxy, oyy, vx, vy, c); break;
                            case 1: adj_fan_view<1, R>(P, base, xmaj, oxx, oyx, oxy, oyy, vx, vy, c); break;
                            default: adj_fan_view<2, R>(P, base, xmaj, oxx, oyx, oxy, oyy, vx, vy, c); break;
                        }
                    }
                    continue;
                }
                const FastRec& P = F;
                const int lo = vab[j].lo;
                // edge views (and every view of a tile with non-finite values):
                // x-major, the forward's inclusion decisions; fixed-point taps into
                // the window, or FP32 taps straight into the sinogram
                const bool direct = any_bad || (G == Geo::kFan && P.mode == kModeEdgeAbs);
                float* Grow = Gs + static_cast<size_t>(ia) * c.ns + lo;
                auto tap = [&](int jj, float sig2, float t) {
                    const float u = __fadd_rn(sig2, -(static_cast<float>(jj - c.kc) - 0.5f));
                    if (direct) {
                        const float a1 = t * u;
                        const int g = lo + jj;  // taps off the detector carry no weight
                        if (t != 0.0f && g >= 0 && g < c.ns) atomicAdd(Grow + jj, t - a1);
                        if (t != 0.0f && g + 1 >= 0 && g + 1 < c.ns) atomicAdd(Grow + jj + 1, a1);
                    } else {
                        const int q1 = static_cast<int>(__float_as_uint(__fmaf_rn(t, u, kMagic)) - kMagicBits);
                        const int q0 = round_int(t) - q1;
                        red_shared_u32(slot + 4u * jj, static_cast<unsigned>(q0));
                        red_shared_u32(slot + 4u * jj + 4u, static_cast<unsigned>(q1));
                    }
                };
                const int iy0 = B.ty0 + warp * R;
                if constexpr (G == Geo::kFan) {
                    if (P.mode == kModeEdgeAbs) {
                        const float x = static_cast<float>(t0[ixx]);
                        for (int r = 0; r < R; ++r) {
                            const int iyc = min(iy0 + r, c.ny - 1);
                            float w, sig2;
                            int jj;
                            const float s = channel_abs<G>(x, static_cast<float>(t1[iyc]), make_float2(P.p0, P.p1), c, &w);
                            if (edge_tap_abs<G>(s, ixx, iyc, ia, lo, t0, t1, t2, c, &jj, &sig2))
                                tap(jj, sig2, (any_bad ? vx[r] : vx[r] * back) * w);
                        }
                        continue;
                    }
                    auto fan_edge = [&](auto vc) {
                        constexpr int V = decltype(vc)::value;
                        const FanX X = fan_xpart(oxx, P);
                        for (int r = 0; r < R; ++r) {
                            float w, sig2;
                            int jj;
                            const float sig = fan_sigma<V>(X, oyx[r], P, c, &w);
                            if (edge_tap<G>(sig, ixx, min(iy0 + r, c.ny - 1), ia, lo, t0, t1, t2, c, &jj, &sig2))
                                tap(jj, sig2, any_bad ? vx[r] * (w * vab[j].e) : __fmul_rn(vx[r], w));
                        }
                    };
                    switch (mode_variant(P.mode)) {
                        case 0: fan_edge(std::integral_constant<int, 0>{}); break;
                        case 1: fan_edge(std::integral_constant<int, 1>{}); break;
                        default: fan_edge(std::integral_constant<int, 2>{}); break;
                    }
                } else {
                    const float xs = par_xpart(oxx, P);
                    for (int r = 0; r < R; ++r) {
                        float sig2;
                        int jj;
                        const float sig = par_sigma(xs, oyx[r], P);
                        if (edge_tap<G>(sig, ixx, min(iy0 + r, c.ny - 1), ia, lo, t0, t1, t2, c, &jj, &sig2))
                            tap(jj, sig2, vx[r]);
                    }
                }
            }
            __syncthreads();
            // flush: window entries -> sinogram (and back to zero); a warp
            // takes whole views, its lanes the window's channels
            for (int j = warp; j < nv; j += kBpThreads / 32) {
                const ViewAux P = vab[j];
                const float sc = back * P.e;
                unsigned* wrow = win + j * c.W;
                float* grow = Gs + static_cast<size_t>(v0 + j) * c.ns + P.lo;
                for (int kk = lane; kk < c.W; kk += 32) {
                    const unsigned a = wrow[kk];
                    if (a == 0u) continue;
                    wrow[kk] = 0u;
                    const int g = P.lo + kk;
                    if (g >= 0 && g < c.ns) atomicAdd(grow + kk, static_cast<float>(static_cast<int>(a)) * sc);
                }
            }
            __syncthreads();
        }
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

// FP32 single-view BP: write-bound (na outputs per pixel).  A CTA owns 32
// consecutive views (one per lane) and a band of image rows; it stages the 32
// sinogram rows in shared memory (row stride odd, so lanes at similar
// channels fall in different banks).  A warp task is a row segment of up to
// kSvSeg pixels: each lane forms its view's channel position at the
// segment's middle pixel in FP64 from the caller's tables (integer part and
// FP32 fraction), then steps through the segment in FP32 with the view's
// slope, so every store of the warp writes 32 consecutive views of one pixel
// (128 contiguous bytes).  The reference's inclusion rule 0 <= s <= ns-1 is
// decided in FP64 (src/bp_par_2d_sv.cc:55-92 arithmetic) for positions within
// a channel of a detector end; farther out the output is 0, farther in the
// FP32 position (within ~4e-6 channels) interpolates.
constexpr int kSvFastThreads = 512;
constexpr int kSvViews = 32;
constexpr int kSvSeg = 64;
constexpr int kSvRowsPerCta = 16;

__global__ void __launch_bounds__(kSvFastThreads, 2)
    bp_par_sv_f32(const float* __restrict__ proj, float* __restrict__ img, const double* __restrict__ xcos,
                  const double* __restrict__ ysin, int ns, int na, int nx, int ny, double ds, double inv_ds,
                  double cents, int stride, size_t proj_stride, size_t img_stride)
{
    extern __shared__ float sv_rows[];  // [kSvViews][stride]
    const int v0 = blockIdx.x * kSvViews;
    const int nv = min(kSvViews, na - v0);
    const float* P = proj + blockIdx.z * proj_stride + static_cast<size_t>(v0) * ns;
    for (int idx = threadIdx.x; idx < nv * ns; idx += kSvFastThreads) {
        const int v = idx / ns, k = idx - v * ns;
        sv_rows[v * stride + k] = __ldg(P + idx);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane >= nv) return;  // no barrier follows
    const int ia = v0 + lane;
    const float* R = sv_rows + lane * stride;
    // the view's channel step per pixel along x, from the caller's x cos t table
    const float px = nx > 1 ? static_cast<float>((xcos[static_cast<size_t>(na) + ia] - xcos[ia]) * inv_ds) : 0.0f;
    float* O = img + blockIdx.z * img_stride + ia;
    const size_t ostep = static_cast<size_t>(na);
    const int y0 = blockIdx.y * kSvRowsPerCta, y1 = min(ny, y0 + kSvRowsPerCta);
    const int segs = (nx + kSvSeg - 1) / kSvSeg;
    for (int task = warp; task < (y1 - y0) * segs; task += kSvFastThreads / 32) {
        const int iy = y0 + task / segs;
        const int xs0 = (task % segs) * kSvSeg, xs1 = min(nx, xs0 + kSvSeg);
        const int xm = (xs0 + xs1) / 2;
        const double ys = ysin[static_cast<size_t>(iy) * na + ia];
        const double sd0 = (xcos[static_cast<size_t>(xm) * na + ia] + ys) * inv_ds + cents;
        const double fl0 = floor(sd0);
        const int i0 = static_cast<int>(fl0);
        // positions less (i0 + 1/2), so that rounding gives the floor
        const float fh = static_cast<float>(sd0 - fl0) - 0.5f;
        float* Or = O + (static_cast<size_t>(iy) * nx + xs0) * ostep;
        // the position is linear along the segment: interior when both ends are
        // at least a channel inside the detector
        const float ka = static_cast<float>(xs0 - xm), kb = static_cast<float>(xs1 - 1 - xm);
        const int ja = i0 + static_cast<int>(floorf(fmaf(ka, px, fh) + 0.5f));
        const int jb = i0 + static_cast<int>(floorf(fmaf(kb, px, fh) + 0.5f));
        if (min(ja, jb) >= 1 && max(ja, jb) <= ns - 3) {
            float kf = ka;
#pragma unroll 4
            for (int ix = xs0; ix < xs1; ++ix, kf += 1.0f, Or += ostep) {
                const float sr = fmaf(kf, px, fh);
                const float vb = __fadd_rn(sr, kMagic);
                const int j = i0 + static_cast<int>(__float_as_uint(vb) - kMagicBits);
                const float u = __fadd_rn(__fadd_rn(sr, -__fadd_rn(vb, -kMagic)), 0.5f);
                const float a = R[j], b = R[j + 1];
                *Or = fmaf(u, b - a, a);
            }
            continue;
        }
        float kf = ka;
        for (int ix = xs0; ix < xs1; ++ix, kf += 1.0f, Or += ostep) {
            const float sr = fmaf(kf, px, fh);
            const float vb = __fadd_rn(sr, kMagic);
            int j = i0 + static_cast<int>(__float_as_uint(vb) - kMagicBits);
            float u = __fadd_rn(__fadd_rn(sr, -__fadd_rn(vb, -kMagic)), 0.5f);
            float out = 0.0f;
            bool in = j >= 1 && j <= ns - 3;
            if (!in && j >= -1 && j <= ns) {
                // within a channel of an end: the reference's FP64 decision
                const double sd = (xcos[static_cast<size_t>(ix) * na + ia] + ys) / ds + cents;
                in = sd >= 0.0 && sd <= static_cast<double>(ns - 1);
                if (in) {
                    const double f = floor(sd);
                    j = static_cast<int>(f);
                    u = static_cast<float>(sd - f);
                }
            }
            if (in) {
                const float a = R[j], b = R[min(j + 1, ns - 1)];
                out = fmaf(u, b - a, a);
            }
            *Or = out;
        }
    }
}

// ---- host side ---------------------------------------------------------------

// Resident CTAs per SM of the tile kernels (two of 256 threads).
constexpr int kTileCtasPerSm = 2;
// Shared memory one tile CTA may take (two CTAs per SM).
constexpr size_t kTileSmemMax = 110 * 1024;

int sm_count() { return device_sms(); }

// Shared bytes of the bulk-copy forward kernel with NG groups of VB views.
inline size_t fwd_smem(const TileConst& ct, int VB, int NG = 1)
{
    const size_t bv = static_cast<size_t>(NG) * VB;
    return 128 + 2 * bv * ct.WS * sizeof(float) + 2 * bv * ct.W * sizeof(float2) + ct.na * kViewBytes;
}

// A backprojection plan's device resources (ctr_bp_plan): stream-K scratch
// whose tile counters (at its start) stay zero between launches, as the CTA
// completing a tile resets its counter, and the geometry's per-(tile, view)
// records (or null: the kernels set them up).
struct BpPlanRes {
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    long long max_tiles = 0;  // counters at the start of scratch
    const FastRec* rec = nullptr;
    const ViewAux* aux = nullptr;
};

// Stream-K launch shape of the bulk-copy kernel for `batch` items: whether it
// applies (fewer than 4 waves of tiles and more than one view block), its CTAs
// and scratch bytes (counters first, then the partial sums).
struct SkShape {
    bool on = false;
    int ctas = 0;
    SkConst k{};
    size_t bytes = 0;
};

template <Geo G, int VB>
SkShape sk_shape(const TileConst& ct, int batch)
{
    SkShape sh;
    const size_t smem = fwd_smem(ct, VB);
    const int tiles_x = static_cast<int>(div_up(ct.nx, kTileX));
    const int tiles_y = static_cast<int>(div_up(ct.ny, kTileY));
    const long long tiles = static_cast<long long>(tiles_x) * tiles_y * batch;
    const int nb = static_cast<int>(div_up(ct.na, VB));
    const int sms = sm_count();
    if (!(tiles < 4ll * sms * kTileCtasPerSm && nb > 1)) return sh;
    auto kern = bp_tile_tma_sk<G, kRowsPerThread, VB, 1, kTileCtasPerSm>;
    int per_sm = 1;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBpThreads, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return sh;
    }
    sh.on = true;
    sh.k.units = tiles * nb;
    sh.k.nb = nb;
    sh.k.tiles_x = tiles_x;
    sh.k.tiles_per_item = tiles_x * tiles_y;
    sh.ctas = static_cast<int>(std::min<long long>(sh.k.units, static_cast<long long>(sms) * per_sm));
    sh.k.maxseg = sk_max_segments(tiles, nb, sh.ctas);
    const size_t counters = (sizeof(int) * static_cast<size_t>(tiles) + 255) & ~static_cast<size_t>(255);
    sh.bytes = counters + static_cast<size_t>(tiles) * sh.k.maxseg * kTileX * kTileY * sizeof(float);
    return sh;
}

// The bulk-copy kernel (one group of VB views, tiles of 32 x kTileY): stream-K
// over (tile, view block) units when the launch has fewer than 4 waves of
// tiles, one CTA per tile otherwise.  With a plan's resources the stream-K
// scratch is the plan's (no allocation, no counter reset) and the view records
// come from its table.
template <Geo G, int VB>
int launch_tma(const float* proj, float* img, const double* t0, const double* t1, const double* t2,
               const TileConst& ct, int batch, cudaStream_t stream, const char* what,
               const BpPlanRes* pr = nullptr)
{
    constexpr int kR = kRowsPerThread;
    const size_t smem = fwd_smem(ct, VB);
    const int tiles_x = static_cast<int>(div_up(ct.nx, kTileX));
    const int tiles_y = static_cast<int>(div_up(ct.ny, kTileY));
    const FastRec* rec = pr ? pr->rec : nullptr;
    const ViewAux* aux = pr ? pr->aux : nullptr;
    SkShape sh = sk_shape<G, VB>(ct, batch);
    if (sh.on) {
        auto kern = bp_tile_tma_sk<G, kR, VB, 1, kTileCtasPerSm>;
        const long long tiles = sh.k.units / sh.k.nb;
        const size_t counters = (sizeof(int) * static_cast<size_t>(tiles) + 255) & ~static_cast<size_t>(255);
        sh.k.rec = rec;
        sh.k.aux = aux;
        const size_t plan_counters =
            pr ? (sizeof(int) * static_cast<size_t>(pr->max_tiles) + 255) & ~static_cast<size_t>(255) : 0;
        if (pr && pr->scratch && tiles <= pr->max_tiles &&
            plan_counters + (sh.bytes - counters) <= pr->scratch_bytes) {
            sh.k.counter = static_cast<int*>(pr->scratch);
            sh.k.partial = reinterpret_cast<float*>(static_cast<char*>(pr->scratch) + plan_counters);
            const cudaError_t e =
                launch_dependent(kern, dim3(sh.ctas), dim3(kBpThreads), smem, stream, proj, img, t0, t1, t2, ct, sh.k);
            if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
            return check_launch(what);
        }
        void* scratch = nullptr;
        if (cudaMallocAsync(&scratch, sh.bytes, stream) == cudaSuccess) {
            sh.k.counter = static_cast<int*>(scratch);
            sh.k.partial = reinterpret_cast<float*>(static_cast<char*>(scratch) + counters);
            cudaError_t e = cudaMemsetAsync(sh.k.counter, 0, sizeof(int) * static_cast<size_t>(tiles), stream);
            if (e == cudaSuccess) {
                kern<<<sh.ctas, kBpThreads, smem, stream>>>(proj, img, t0, t1, t2, ct, sh.k);
                e = cudaGetLastError();
            }
            cudaFreeAsync(scratch, stream);
            if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
            return CTR_OK;
        }
        cudaGetLastError();  // no scratch: whole tiles per CTA below
    }
    auto kern = bp_tile_tma_f32<G, kR, kTileCtasPerSm, VB, 1>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    dim3 grid(tiles_x, tiles_y, batch);
    e = launch_dependent(kern, grid, dim3(kBpThreads), smem, stream, proj, img, t0, t1, t2, ct, rec, aux);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return check_launch(what);
}

// Forward dispatch: the bulk-copy kernel when its window fits one 256-element
// box and the sinogram is 16-byte aligned (parallel: 32 views per block where
// that fits the shared memory, else 16), the cooperative kernel otherwise.
// Both use the geometry's one window (c.W), so they compute the same
// positions as the adjoint.
template <Geo G>
int launch_forward(const float* proj, float* img, const double* t0, const double* t1,
                   const double* t2, TileConst c, int batch, cudaStream_t stream, const char* what,
                   const BpPlanRes* pr = nullptr)
{
    const unsigned long long total = static_cast<unsigned long long>(c.proj_stride) * batch;
    c.total4 = static_cast<long long>(total & ~3ull);
    if (c.WB <= 256 && reinterpret_cast<uintptr_t>(proj) % 16 == 0 && total < (1ull << 31) &&
        c.na <= 4096) {
        // parallel: 32 views per block halve the block barriers of its short
        // per-view work; the fan keeps 16
        if (G == Geo::kPar && fwd_smem(c, 32) <= kTileSmemMax)
            return launch_tma<G, 32>(proj, img, t0, t1, t2, c, batch, stream, what, pr);
        if (fwd_smem(c, 16) <= kTileSmemMax)
            return launch_tma<G, 16>(proj, img, t0, t1, t2, c, batch, stream, what, pr);
    }
    const size_t smem = static_cast<size_t>(kViewBlock) * c.W * sizeof(float2);
    if (smem > 160 * 1024) return fail(CTR_ERR_UNSUPPORTED, "%s: window of %d channels too wide", what, c.W);
    auto kern = bp_tile_f32_coop<G>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    dim3 grid(div_up(c.nx, kTileX), div_up(c.ny, kTileY), batch);
    kern<<<grid, kBpThreads, smem, stream>>>(proj, img, t0, t1, t2, c);
    return check_launch(what);
}

// Fixed-point bits of the adjoint's largest tap: a window entry sums the taps
// of the tile's pixels within one channel of it, at most `hits` pixels (a
// band two channel pitches wide across the tile, on the pixel lattice), each
// below 2^(fx_bits+1) (the fan's relative weight is at most ~2); the sum must
// stay below 2^31.
int adj_fx_bits(double pitch_mm, double dx, double dy)
{
    const double pix = std::min(std::fabs(dx), std::fabs(dy));
    const double diag = std::sqrt(std::pow(kTileX * dx, 2) + std::pow(kTileY * dy, 2)) / pix;
    double hits = (2.0 * std::fabs(pitch_mm) / pix + 1.5) * (diag + 1.5);
    if (!(hits < kTileX * kTileY)) hits = kTileX * kTileY;
    int fx = 20;
    while (fx > 8 && hits * std::ldexp(2.0, fx) >= 2147483647.0) --fx;
    return fx;
}

// The adjoint: stream-K over (tile, view block) units, as many CTAs as are
// resident.
template <Geo G>
int launch_adjoint(const float* img, float* grad, const double* t0, const double* t1, const double* t2,
                   const TileConst& c, int batch, cudaStream_t stream, const char* what,
                   const BpPlanRes* pr = nullptr)
{
    const size_t smem = (static_cast<size_t>(kViewBlock) * c.W * 4 + 15) / 16 * 16 +
                        static_cast<size_t>(kAdjChunkBlocks * kViewBlock) * kViewBytes;
    if (smem > kTileSmemMax) return fail(CTR_ERR_UNSUPPORTED, "%s: window of %d channels too wide", what, c.W);
    const int tiles_x = static_cast<int>(div_up(c.nx, kTileX));
    const int tiles_y = static_cast<int>(div_up(c.ny, kTileY));
    AdjUnits k{};
    k.nb = static_cast<int>(div_up(c.na, kViewBlock));
    k.tiles_x = tiles_x;
    k.tiles_per_item = tiles_x * tiles_y;
    k.units = static_cast<long long>(k.tiles_per_item) * batch * k.nb;
    k.rec = pr ? pr->rec : nullptr;
    k.aux = pr ? pr->aux : nullptr;
    auto kern = bp_tile_adj<G>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    int per_sm = 1;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBpThreads, smem);
    if (e != cudaSuccess || per_sm < 1) return fail(CTR_ERR_CUDA, "%s: occupancy", what);
    const int ctas = static_cast<int>(std::min<long long>(k.units, static_cast<long long>(sm_count()) * per_sm));
    kern<<<ctas, kBpThreads, smem, stream>>>(img, grad, t0, t1, t2, c, k);
    return check_launch(what);
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

// The FP32 kernels' constants for a fan geometry (window for 32 x kTileY tiles).
TileConst fan_const(const FanArgs& a, double extra_scale)
{
    TileConst c{};
    c.ns = a.ns; c.na = a.na; c.nx = a.nx; c.ny = a.ny;
    set_window(c, tile_window(fan_window(a.ns, a.ds, a.dso, a.dsd, a.nx, a.ny, a.dx, a.dy, a.offset_x,
                                         a.offset_y)));
    c.cents = static_cast<float>((a.ns - 1) / 2.0 + a.offset_s);
    c.nsm1 = static_cast<float>(a.ns - 1);
    c.dso = static_cast<float>(a.dso);
    c.K = static_cast<float>(a.dsd / a.ds);
    c.scale = static_cast<float>(a.dsd * a.dsd * extra_scale);
    c.dx = a.dx;
    c.dy = a.dy;
    c.dxf = static_cast<float>(a.dx);
    c.dyf = static_cast<float>(a.dy);
    c.ds_d = a.ds;
    c.cents_d = (a.ns - 1) / 2.0 + a.offset_s;
    c.dso_d = a.dso;
    c.dsd_d = a.dsd;
    fill_fan_tables(c, a.dsd, a.ds);
    // channel pitch at the far side of the image (the widest)
    const double hx = ((a.nx - 1) / 2.0 + std::fabs(a.offset_x)) * a.dx;
    const double hy = ((a.ny - 1) / 2.0 + std::fabs(a.offset_y)) * a.dy;
    c.fx_bits = adj_fx_bits(a.ds * (std::fabs(a.dso) + std::sqrt(hx * hx + hy * hy)) / std::fabs(a.dsd), a.dx, a.dy);
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
        const TileConst c = fan_const(a, scaled ? a.scale : 1.0);
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
        const TileConst c = fan_const(a, scaled ? a.scale : 1.0);
        return launch_adjoint<Geo::kFan>(img, grad, xpos, ypos, sc, c, batch, stream, "bp_fan_2d_grad");
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

// The FP32 kernels' constants for a parallel geometry (window for 32 x kTileY tiles).
TileConst par_const(const ctr_par_param* p)
{
    TileConst c{};
    c.ns = p->ns; c.na = p->na; c.nx = p->nx; c.ny = p->ny;
    set_window(c, tile_window(par_window(p->ns, p->ds, p->dx, p->dy)));
    c.cents = static_cast<float>((p->ns - 1) / 2.0 + p->offset_s);
    c.nsm1 = static_cast<float>(p->ns - 1);
    c.scale = static_cast<float>(p->orbit);
    c.orbit_start = p->orbit_start;
    c.orbit = p->orbit;
    c.inv_ds = 1.0 / p->ds;
    c.inv_dx = 1.0 / p->dx;
    c.inv_dy = 1.0 / p->dy;
    c.centx = (p->nx - 1) / 2.0 + p->offset_x;
    c.centy = (p->ny - 1) / 2.0 + p->offset_y;
    c.dx = p->dx;
    c.dy = p->dy;
    c.dxf = static_cast<float>(p->dx);
    c.dyf = static_cast<float>(p->dy);
    c.ds_d = p->ds;
    c.cents_d = (p->ns - 1) / 2.0 + p->offset_s;
    c.fx_bits = adj_fx_bits(p->ds, p->dx, p->dy);
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
        return launch_forward<Geo::kPar>(proj, img, xcos, ysin, nullptr, par_const(p), batch, stream,
                                         "bp_par_2d");
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
        return launch_adjoint<Geo::kPar>(img, grad, xcos, ysin, nullptr, par_const(p), batch, stream,
                                         "bp_par_2d_grad");
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
    if constexpr (sizeof(T) == 4) {
        const int stride = static_cast<int>(p->ns) | 1;
        const size_t smem = sizeof(float) * kSvViews * static_cast<size_t>(stride);
        if (smem <= 220 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(bp_par_sv_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(smem));
            if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "bp_par_2d_sv: %s", cudaGetErrorString(e));
            dim3 g2(div_up(p->na, kSvViews), div_up(p->ny, kSvRowsPerCta), batch);
            bp_par_sv_f32<<<g2, kSvFastThreads, smem, stream>>>(
                proj, img, xcos, ysin, p->ns, p->na, p->nx, p->ny, p->ds, 1.0 / p->ds, cents, stride,
                static_cast<size_t>(p->ns) * p->na, static_cast<size_t>(p->nx) * p->ny * p->na);
            return check_launch("bp_par_2d_sv");
        }
    }
    dim3 grid(div_up(p->nx, kSvPix), p->ny, batch);
    bp_par_sv<T><<<grid, kSvThreads, 0, stream>>>(proj, img, xcos, ysin, p->ns, p->na, p->nx,
                                                  p->ny, p->ds, cents,
                                                  static_cast<size_t>(p->ns) * p->na,
                                                  static_cast<size_t>(p->nx) * p->ny * p->na);
    return check_launch("bp_par_2d_sv");
}

// Largest record table a plan keeps (beyond it the kernels set views up).
constexpr size_t kBpPlanRecMax = 64ull << 20;

}  // namespace
}  // namespace ctr

// A backprojection plan: the geometry's tables (copies), the constants, the
// stream-K scratch and the per-(tile, view) records, for the FP32 forward.
struct ctr_bp_plan {
    int device = 0;
    int max_batch = 0;
    bool fan = false;
    ctr::TileConst c{};
    double* tabs = nullptr;
    const double* t0 = nullptr;
    const double* t1 = nullptr;
    const double* t2 = nullptr;
    ctr::BpPlanRes res{};
    void* rec_mem = nullptr;
    ~ctr_bp_plan()
    {
        if (tabs) cudaFree(tabs);
        if (res.scratch) cudaFree(res.scratch);
        if (rec_mem) cudaFree(rec_mem);
    }
};

namespace ctr {
namespace {

// The view block the forward dispatch picks for a geometry (0: not the
// bulk-copy kernels).
template <Geo G>
int plan_view_block(const TileConst& c)
{
    if (!(c.WB <= 256 && c.na <= 4096)) return 0;
    if (G == Geo::kPar && fwd_smem(c, 32) <= kTileSmemMax) return 32;
    return fwd_smem(c, 16) <= kTileSmemMax ? 16 : 0;
}

template <Geo G, int VB>
void plan_scratch_need(const TileConst& c, int max_batch, long long* max_tiles, size_t* part_max)
{
    for (int b = 1; b <= max_batch; ++b) {
        const SkShape sh = sk_shape<G, VB>(c, b);
        if (!sh.on) continue;
        const long long tiles = sh.k.units / sh.k.nb;
        const size_t counters = (sizeof(int) * static_cast<size_t>(tiles) + 255) & ~static_cast<size_t>(255);
        *max_tiles = std::max(*max_tiles, tiles);
        *part_max = std::max(*part_max, sh.bytes - counters);
    }
}

// Copies the tables (n[i] doubles from src[i]), sizes and zeroes the stream-K
// scratch for every batch up to max_batch, and writes the records.
template <Geo G>
int bp_plan_make(ctr_bp_plan* P, const double* const src[3], const size_t n[3], cudaStream_t stream)
{
    const size_t total = n[0] + n[1] + n[2];
    if (cudaMalloc(&P->tabs, total * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return fail(CTR_ERR_CUDA, "bp plan: %zu bytes of tables", total * sizeof(double));
    }
    size_t off = 0;
    const double** dst[3] = {&P->t0, &P->t1, &P->t2};
    for (int i = 0; i < 3; ++i) {
        *dst[i] = n[i] ? P->tabs + off : nullptr;
        if (n[i] && cudaMemcpyAsync(P->tabs + off, src[i], n[i] * sizeof(double), cudaMemcpyDeviceToDevice,
                                    stream) != cudaSuccess)
            return fail(CTR_ERR_CUDA, "bp plan: table copy");
        off += n[i];
    }
    const TileConst& c = P->c;
    const int vb = plan_view_block<G>(c);
    if (vb == 0) return cudaStreamSynchronize(stream) == cudaSuccess ? CTR_OK : fail(CTR_ERR_CUDA, "bp plan");
    long long max_tiles = 0;
    size_t part = 0;
    if (vb == 32) plan_scratch_need<G, 32>(c, P->max_batch, &max_tiles, &part);
    else plan_scratch_need<G, 16>(c, P->max_batch, &max_tiles, &part);
    if (max_tiles > 0) {
        const size_t counters = (sizeof(int) * static_cast<size_t>(max_tiles) + 255) & ~static_cast<size_t>(255);
        if (cudaMalloc(&P->res.scratch, counters + part) != cudaSuccess ||
            cudaMemsetAsync(P->res.scratch, 0, counters, stream) != cudaSuccess) {
            cudaGetLastError();
            return fail(CTR_ERR_CUDA, "bp plan: %zu bytes of scratch", counters + part);
        }
        P->res.scratch_bytes = counters + part;
        P->res.max_tiles = max_tiles;
    }
    const int tiles_x = static_cast<int>(div_up(c.nx, kTileX));
    const int tiles = tiles_x * static_cast<int>(div_up(c.ny, kTileY));
    const size_t nrec = static_cast<size_t>(tiles) * c.na;
    if (nrec * kViewBytes <= kBpPlanRecMax) {
        if (cudaMalloc(&P->rec_mem, nrec * kViewBytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(CTR_ERR_CUDA, "bp plan: %zu bytes of view records", nrec * kViewBytes);
        }
        FastRec* rec = static_cast<FastRec*>(P->rec_mem);
        ViewAux* aux = reinterpret_cast<ViewAux*>(rec + nrec);
        const unsigned blocks = static_cast<unsigned>(std::min<size_t>(div_up(nrec, 256), 8ull * sm_count()));
        bp_view_records<G><<<blocks, 256, 0, stream>>>(P->t0, P->t1, P->t2, c, tiles_x, tiles, rec, aux);
        const int st = check_launch("bp plan records");
        if (st) return st;
        P->res.rec = rec;
        P->res.aux = aux;
    }
    const cudaError_t e = cudaStreamSynchronize(stream);
    return e == cudaSuccess ? CTR_OK : fail(CTR_ERR_CUDA, "bp plan set-up: %s", cudaGetErrorString(e));
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_bp_par_2d_plan_create(const ctr_par_param* p, const double* xcos, const double* ysin, int max_batch,
                              ctr_bp_plan** plan, cudaStream_t stream)
{
    if (!plan) return fail(CTR_ERR_INVALID_ARG, "null plan pointer");
    *plan = nullptr;
    int st = check_par(p, xcos, ysin, xcos, ysin, max_batch);
    if (st) return st;
    auto P = std::make_unique<ctr_bp_plan>();
    cudaGetDevice(&P->device);
    P->max_batch = max_batch;
    P->fan = false;
    P->c = par_const(p);
    const double* src[3] = {xcos, ysin, nullptr};
    const size_t n[3] = {static_cast<size_t>(p->nx) * p->na, static_cast<size_t>(p->ny) * p->na, 0};
    st = bp_plan_make<Geo::kPar>(P.get(), src, n, stream);
    if (st) return st;
    *plan = P.release();
    return CTR_OK;
}

int ctr_bp_fan_2d_plan_create(const ctr_fan_bp_param* p, const double* xpos, const double* ypos,
                              const double* sincostbl, int max_batch, ctr_bp_plan** plan,
                              cudaStream_t stream)
{
    if (!plan) return fail(CTR_ERR_INVALID_ARG, "null plan pointer");
    *plan = nullptr;
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null argument");
    const FanArgs a = fan_args(p);
    int st = check_fan(a, xpos, ypos, xpos, ypos, sincostbl, max_batch);
    if (st) return st;
    auto P = std::make_unique<ctr_bp_plan>();
    cudaGetDevice(&P->device);
    P->max_batch = max_batch;
    P->fan = true;
    P->c = fan_const(a, a.scale);
    const double* src[3] = {xpos, ypos, sincostbl};
    const size_t n[3] = {p->nx, p->ny, 2 * static_cast<size_t>(p->na)};
    st = bp_plan_make<Geo::kFan>(P.get(), src, n, stream);
    if (st) return st;
    *plan = P.release();
    return CTR_OK;
}

int ctr_bp_plan_run(ctr_bp_plan* plan, const float* proj, float* img, int batch, cudaStream_t stream)
{
    if (!plan || !proj || !img) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != plan->device) return fail(CTR_ERR_INVALID_ARG, "plan made on device %d, current %d", plan->device, dev);
    if (batch > plan->max_batch) return fail(CTR_ERR_INVALID_ARG, "batch %d > the plan's %d", batch, plan->max_batch);
    if (plan->fan)
        return launch_forward<Geo::kFan>(proj, img, plan->t0, plan->t1, plan->t2, plan->c, batch, stream,
                                         "bp_fan_2d", &plan->res);
    return launch_forward<Geo::kPar>(proj, img, plan->t0, plan->t1, plan->t2, plan->c, batch, stream, "bp_par_2d",
                                     &plan->res);
}

int ctr_bp_plan_run_grad(ctr_bp_plan* plan, const float* img, float* grad, int batch, cudaStream_t stream)
{
    if (!plan || !img || !grad) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != plan->device) return fail(CTR_ERR_INVALID_ARG, "plan made on device %d, current %d", plan->device, dev);
    if (batch > plan->max_batch) return fail(CTR_ERR_INVALID_ARG, "batch %d > the plan's %d", batch, plan->max_batch);
    const cudaError_t e = cudaMemsetAsync(grad, 0, sizeof(float) * plan->c.proj_stride * batch, stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "zero grad: %s", cudaGetErrorString(e));
    if (plan->fan)
        return launch_adjoint<Geo::kFan>(img, grad, plan->t0, plan->t1, plan->t2, plan->c, batch, stream,
                                         "bp_fan_2d_grad", &plan->res);
    return launch_adjoint<Geo::kPar>(img, grad, plan->t0, plan->t1, plan->t2, plan->c, batch, stream,
                                     "bp_par_2d_grad", &plan->res);
}

int ctr_bp_plan_destroy(ctr_bp_plan* plan)
{
    delete plan;
    return CTR_OK;
}


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
