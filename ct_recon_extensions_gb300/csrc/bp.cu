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
// shared memory as pairs, zero outside the detector: (p[k] - k d[k], d[k]),
// d[k] = p[k+1] - p[k], k the channel less the window start, in the TMA-fed
// kernels, (p[k], d[k]) in the plain one.  A pixel-view update is then:
// channel position (relative to the window start), its floor, one 8-byte
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
#include <type_traits>

#include "bp_tile.cuh"

namespace ctr {
namespace {

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
    extern __shared__ __align__(16) float accw[];  // [kViewBlock][W], then ViewT<G>[na]
    ViewT<G>* views = reinterpret_cast<ViewT<G>*>(accw + (kViewBlock * c.W + 3) / 4 * 4);

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
    // per-view parameters, windows and paths of this tile for the whole scan
    for (int ia = threadIdx.x; ia < c.na; ia += kBpThreads)
        views[ia] = view_setup<G>(t0, t1, t2, ia, tx0, ty0, cx0, cx1, cy0, cy1, c);

    for (int v0 = 0; v0 < c.na; v0 += kViewBlock) {
        const int nv = min(kViewBlock, c.na - v0);
        for (int idx = threadIdx.x; idx < nv * c.W; idx += kBpThreads) accw[idx] = 0.0f;
        __syncthreads();
        for (int j = 0; j < nv; ++j) {
            const ViewT<G> P = views[v0 + j];
            float* aj = accw + j * c.W;
            if (mode_fast(P.mode)) {
                const float cen = view_cen<G>(P, c);
                float xs, xc;
                fast_xs<G>(fast_coord<G>(x, cx0), P.vp, cen, c, &xs, &xc);
                auto taps = [&](auto variant) {
                    constexpr int V = decltype(variant)::value;
#pragma unroll
                    for (int r = 0; r < kRowsPerThread; ++r) {
                        float w;
                        const float s = fast_s<G, V>(xs, xc, fast_coord<G>(y[r], cy0), P.vp, cen, c, &w);  // s - lo
                        const float v = s + kMagicHalf;
                        const float u = s - (v - kMagic);
                        const int k = static_cast<int>(__float_as_uint(v) - kMagicBits);
                        const float t = val[r] * w;
                        if (t != 0.0f) {
                            atomicAdd(aj + k, t - t * u);
                            atomicAdd(aj + k + 1, t * u);
                        }
                    }
                };
                switch (G == Geo::kFan ? P.mode & 3 : 0) {
                    case 0: taps(std::integral_constant<int, 0>{}); break;
                    case 1: taps(std::integral_constant<int, 1>{}); break;
                    case 2: taps(std::integral_constant<int, 2>{}); break;
                    default: taps(std::integral_constant<int, 3>{}); break;
                }
            } else if (P.mode == kModeEdge) {
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
            const int g = views[v0 + j].lo + k;
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

template <class K>
int launch_tile(K kern, int W, dim3 grid, cudaStream_t stream, const char* what,
                const void* a0, void* a1, const double* xpos, const double* ypos,
                const double* sincos, const TileConst& c, bool adjoint)
{
    size_t smem = static_cast<size_t>(kViewBlock) * W * (adjoint ? sizeof(float) : sizeof(float2));
    if (adjoint) smem = (static_cast<size_t>(kViewBlock) * W + 3) / 4 * 4 * sizeof(float) + c.na * kViewBytesMax;
    if (smem > 160 * 1024) return fail(CTR_ERR_UNSUPPORTED, "%s: window of %d channels too wide", what, W);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    kern<<<grid, kBpThreads, smem, stream>>>(static_cast<const float*>(a0), static_cast<float*>(a1),
                                             xpos, ypos, sincos, c);
    return check_launch(what);
}


// Rows per thread of the bulk-copy forward kernel (tile 32 x 8*kFwdRows) and
// its resident CTAs per SM (sets the register budget).
constexpr int kFwdRows = 8;
constexpr int kFwdMinBlocks = 1;
// View groups per CTA of the single-geometry forward kernel: 2 (512 threads,
// one CTA per SM) or 1 (256 threads, two CTAs per SM on different tiles).
constexpr int kFwdGroups = 1;
constexpr int kFwdTileY = (kBpThreads / 32) * kFwdRows;
// Shared memory the forward kernel may take (one CTA per SM).
constexpr size_t kFwdSmemMax = 200 * 1024;

// Shared bytes of the bulk-copy forward kernel with NG groups of VB views.
template <Geo G>
inline size_t fwd_smem(const TileConst& ct, int VB, int NG = kGroups)
{
    const size_t bv = static_cast<size_t>(NG) * VB;
    return 128 + 2 * bv * ct.WS * sizeof(float) + 2 * bv * ct.W * sizeof(float2) + ct.na * sizeof(ViewT<G>);
}

// The bulk-copy kernel with VB views per group on tiles of 32 x kFwdTileY:
// stream-K over (tile, view block) units when the launch has fewer than 4
// waves of tiles, one CTA per tile otherwise.
template <Geo G, int VB, int NG>
int launch_tma(const float* proj, float* img, const double* t0, const double* t1, const double* t2,
               const TileConst& ct, int batch, cudaStream_t stream, const char* what)
{
    constexpr int kThreads = NG * kBpThreads;
    constexpr int kMinBlocks = NG == 1 ? 2 : kFwdMinBlocks;  // same register budget per SM
    const size_t smem = fwd_smem<G>(ct, VB, NG);
    const int tiles_x = static_cast<int>(div_up(ct.nx, kTileX));
    const int tiles_y = static_cast<int>(div_up(ct.ny, kFwdTileY));
    const long long tiles = static_cast<long long>(tiles_x) * tiles_y * batch;
    const int nb = static_cast<int>(div_up(ct.na, NG * VB));
    int dev = 0, sms = kSmCount;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (tiles < 4ll * sms * kMinBlocks && nb > 1) {
        SkConst k{};
        k.units = tiles * nb;
        k.nb = nb;
        k.tiles_x = tiles_x;
        k.tiles_per_item = tiles_x * tiles_y;
        auto kern = bp_tile_tma_sk<G, kFwdRows, VB, NG, kMinBlocks>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        int per_sm = 1;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
        if (e != cudaSuccess || per_sm < 1) return fail(CTR_ERR_CUDA, "%s: occupancy", what);
        const int ctas = static_cast<int>(std::min<long long>(k.units, static_cast<long long>(sms) * per_sm));
        k.maxseg = sk_max_segments(tiles, nb, ctas);
        const size_t part_bytes = static_cast<size_t>(tiles) * k.maxseg * kTileX * kFwdTileY * sizeof(float);
        void* scratch = nullptr;
        if (cudaMallocAsync(&scratch, part_bytes + sizeof(int) * tiles, stream) == cudaSuccess) {
            k.partial = static_cast<float*>(scratch);
            k.counter = reinterpret_cast<int*>(static_cast<char*>(scratch) + part_bytes);
            e = cudaMemsetAsync(k.counter, 0, sizeof(int) * tiles, stream);
            if (e == cudaSuccess) {
                kern<<<ctas, kThreads, smem, stream>>>(proj, img, t0, t1, t2, ct, k);
                e = cudaGetLastError();
            }
            cudaFreeAsync(scratch, stream);
            if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
            return CTR_OK;
        }
        cudaGetLastError();  // no scratch: whole tiles per CTA below
    }
    auto kern = bp_tile_tma_f32<G, kFwdRows, kMinBlocks, VB, NG>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    dim3 grid(tiles_x, tiles_y, batch);
    kern<<<grid, kThreads, smem, stream>>>(proj, img, t0, t1, t2, ct);
    return check_launch(what);
}

// Forward dispatch: the bulk-copy kernel (tile 32 x kFwdTileY, window w_tall;
// parallel: 32 views per group where that fits the shared memory, else 16) when its
// window fits 256 elements and the sinogram is 16-byte aligned, the
// cooperative kernel (tile 32 x kTileY, window c.W) otherwise.
template <Geo G>
int launch_forward(const float* proj, float* img, const double* t0, const double* t1,
                   const double* t2, TileConst c, int w_tall, int batch, cudaStream_t stream,
                   const char* what)
{
    TileConst ct = c;
    // the final group reduction reuses one half of the pair buffer (2*VB x W
    // float2) for kFwdRows x kBpThreads floats: W >= 4 * kFwdRows (VB >= 16)
    ct.W = std::max({w_tall, 16, kFwdRows * kBpThreads / (2 * kBlockViews)});
    ct.WB = (ct.W + 4 + 3) / 4 * 4;
    ct.WS = (ct.WB + 31) / 32 * 32;
    const unsigned long long total = static_cast<unsigned long long>(c.proj_stride) * batch;
    ct.total4 = static_cast<long long>(total & ~3ull);
    if (ct.WB <= 256 && reinterpret_cast<uintptr_t>(proj) % 16 == 0 && total < (1ull << 31) &&
        c.na <= 4096) {
        // parallel: 32 views per group halve the block barriers of its short
        // per-view work (bp_par_2d 122.9 -> 121.7 us at 512^2); the fan keeps 16
        // (183 vs 190 us with 32)
        if (G == Geo::kPar && fwd_smem<G>(ct, 32, kFwdGroups) <= kFwdSmemMax / (3 - kFwdGroups))
            return launch_tma<G, 32, kFwdGroups>(proj, img, t0, t1, t2, ct, batch, stream, what);
        if (fwd_smem<G>(ct, 16, kFwdGroups) <= kFwdSmemMax / (3 - kFwdGroups))
            return launch_tma<G, 16, kFwdGroups>(proj, img, t0, t1, t2, ct, batch, stream, what);
    }
    c.W = std::max(c.W, 16);
    dim3 grid(div_up(c.nx, kTileX), div_up(c.ny, kTileY), batch);
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
    for (int v = 0; v < kAtanVariants; ++v)
        for (int k = 0; k < 6; ++k) c.poly[v][k] = static_cast<float>(kAtanPoly[v][k] * a.dsd / a.ds);
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
        const int w_tall = fan_window(a.ns, a.ds, a.dso, a.dsd, a.nx, a.ny, a.dx, a.dy, a.offset_x,
                                      a.offset_y, kFwdTileY);
        return launch_forward<Geo::kFan>(proj, img, xpos, ypos, sc, c, w_tall, batch, stream, "bp_fan_2d");
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
        const int w_tall = par_window(p->ns, p->ds, p->dx, p->dy, kFwdTileY);
        return launch_forward<Geo::kPar>(proj, img, xcos, ysin, nullptr, c, w_tall, batch, stream,
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
