// Parallel-beam ray-driven forward projection and its adjoint (reference
// src/fp_par_2d.cc:210-391).
//
// Views whose rays run closer to the y axis (usex) march image rows and
// interpolate along x; the others march columns and interpolate along y.  A
// sample is included iff its fractional index lies in [0, n-1], the
// reference's CPU rule (src/fp_par_2d.cc:237,259); the ray sum is scaled by
// dy/|cos| or dx/|sin|.
//
// FP32 forward: a CTA owns a few consecutive views and all their channels; it
// streams the image through shared memory in bands of rows (or of columns,
// stored transposed) that every ray of the CTA reads, so global reads are
// coalesced and each image byte is fetched from L2 once per CTA.  Each ray's
// sample range is decided once in FP64; positions are 32.32 fixed point, so
// a sample costs one 64-bit add, the fraction and an 8-byte shared read pair.
//
// FP32 adjoint: one thread per pixel gathers, for every view, the channels of
// its footprint with the triangle weights of the reference's grad
// (src/fp_par_2d.cc:339-383), channel positions in 32.32 fixed point from the
// caller's grad-prep table.  The channel range is clamped to the detector
// (the reference reads without a bounds check there).  No atomics.
//
// FP64 kernels follow the reference's arithmetic (one thread per ray / pixel).
#include <algorithm>
#include <mutex>

#include "ctr_async.cuh"
#include "ctr_common.cuh"

namespace ctr {
namespace {

// ---- FP32 forward: image bands in shared memory, fixed-point sample positions

constexpr int kFpThreads = 512;
constexpr int kFpMaxRays = 8;  // rays per thread
// Sample positions are 32.32 fixed point.  Each ray's line X(k) = X0 + k*S is
// anchored at its smallest-x valid sample, X(anchor) = round(x(anchor) * 2^32)
// >= 0, and is monotonic along the ray, so X >= 0 on every valid sample and its
// integer part is a valid pixel index; rounding S moves a position by at most
// |k - anchor|/2 units (< 6e-8 px for 512 samples).
constexpr double kTwo32 = 4294967296.0;

// 32.32 fixed-point line of a ray with FP64 start/step over samples [k0, k1].
__device__ __forceinline__ long long ray_line(double begin, double step, int k0, int k1, long long* S)
{
    *S = llrint(step * kTwo32);
    const int ka = step < 0.0 ? k1 : k0;  // smallest x
    return llrint(fma(static_cast<double>(ka), step, begin) * kTwo32) - static_cast<long long>(ka) * *S;
}

struct FpConst {
    int ns, na, nx, ny;
    int views;  // views per CTA
    int band;   // staged lines per band
    double dx, dy;
    size_t img_stride, proj_stride;
};

__device__ __forceinline__ float frac_of(long long X)
{
    return __uint_as_float(0x3F800000u | (static_cast<unsigned>(X) >> 9)) - 1.0f;
}

// Sample range [k0, k1] of a ray with FP64 start/step: 0 <= begin + k*step <= lim
// (the reference's inclusion rule, src/fp_par_2d.cc:237).
__device__ void ray_range(double begin, double step, int nsamp, int lim, int* k0o, int* k1o)
{
    int k0 = 0, k1 = nsamp - 1;
    if (step == 0.0) {
        if (!(begin >= 0.0 && begin <= lim)) k1 = -1;
    } else {
        double a = (0.0 - begin) / step, b = (lim - begin) / step;
        if (a > b) {
            const double t = a;
            a = b;
            b = t;
        }
        k0 = max(k0, static_cast<int>(fmax(ceil(a), -1.0)));
        k1 = min(k1, static_cast<int>(fmin(floor(b), static_cast<double>(nsamp))));
        if (k0 <= k1) {  // settle the divisions' rounding on the samples themselves
            const double xa = fma(static_cast<double>(k0), step, begin);
            if (!(xa >= 0.0 && xa <= lim)) {
                ++k0;
            } else if (k0 > 0) {
                const double xp = fma(static_cast<double>(k0 - 1), step, begin);
                if (xp >= 0.0 && xp <= lim) --k0;
            }
        }
        if (k0 <= k1) {
            const double xb = fma(static_cast<double>(k1), step, begin);
            if (!(xb >= 0.0 && xb <= lim)) {
                --k1;
            } else if (k1 < nsamp - 1) {
                const double xn = fma(static_cast<double>(k1 + 1), step, begin);
                if (xn >= 0.0 && xn <= lim) ++k1;
            }
        }
    }
    *k0o = k0;
    *k1o = k1;
}

// A CTA projects `views` consecutive views (all channels).  Rays of row-marching
// views (usex) and of column-marching views are run in separate passes; each
// pass stages the image in bands of `band` rows (or columns, stored transposed)
// that all rays of the pass read from shared memory.
__global__ void __launch_bounds__(kFpThreads)
    fp_band_f32(const float* __restrict__ img, float* __restrict__ proj,
                const double* __restrict__ sincos, const double* __restrict__ bo,
                const int* __restrict__ usex, const FpConst c)
{
    extern __shared__ float band[];  // [band][len + 1]
    const int v0 = blockIdx.x * c.views;
    const int nv = min(c.views, c.na - v0);
    const int nrays = nv * c.ns;
    const float* I = img + blockIdx.y * c.img_stride;

    long long X[kFpMaxRays], S[kFpMaxRays];
    int k0[kFpMaxRays], k1[kFpMaxRays], cls[kFpMaxRays];
    float sum[kFpMaxRays];
    bool has_cls[2] = {false, false};
#pragma unroll
    for (int j = 0; j < kFpMaxRays; ++j) {
        const int r = threadIdx.x + j * kFpThreads;
        sum[j] = 0.0f;
        cls[j] = -1;
        X[j] = 0;
        S[j] = 0;
        k0[j] = 0;
        k1[j] = -1;
        if (r < nrays) {
            const int ia = v0 + r / c.ns;
            const size_t ray = static_cast<size_t>(v0) * c.ns + r;
            const int ux = usex[ia] != 0;
            const double begin = bo[2 * ray], step = bo[2 * ray + 1];
            const int nsamp = ux ? c.ny : c.nx;
            const int lim = ux ? c.nx - 1 : c.ny - 1;
            ray_range(begin, step, nsamp, lim, &k0[j], &k1[j]);
            X[j] = ray_line(begin, step, k0[j], k1[j], &S[j]);
            cls[j] = ux ? 0 : 1;
            has_cls[cls[j]] = true;
        }
    }
    for (int pass = 0; pass < 2; ++pass) {
        if (!__syncthreads_or(has_cls[pass])) continue;
        const int n = pass == 0 ? c.ny : c.nx;    // samples along the ray
        const int len = pass == 0 ? c.nx : c.ny;  // staged line length
        const int ld = len + 1;                   // zero pad after each line
        for (int b0 = 0; b0 < n; b0 += c.band) {
            const int nb = min(c.band, n - b0);
            if (pass == 0) {
                for (int idx = threadIdx.x; idx < nb * ld; idx += kFpThreads) {
                    const int i = idx / ld, t = idx - i * ld;
                    band[idx] = t < len ? __ldg(I + static_cast<size_t>(b0 + i) * c.nx + t) : 0.0f;
                }
            } else {
                // column band: read rows of nb consecutive pixels, store transposed
                for (int idx = threadIdx.x; idx < nb * ld; idx += kFpThreads) {
                    const int t = idx / nb, i = idx - t * nb;
                    band[i * ld + t] = t < len ? __ldg(I + static_cast<size_t>(t) * c.nx + b0 + i) : 0.0f;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kFpMaxRays; ++j) {
                if (cls[j] != pass) continue;
                const int ka = max(k0[j], b0), kb = min(k1[j], b0 + nb - 1);
                if (ka > kb) continue;
                long long x = X[j] + static_cast<long long>(ka) * S[j];
                const float* line = band + (ka - b0) * ld;
                float acc = 0.0f;  // this band's partial sum (blocked summation)
                for (int k = ka; k <= kb; ++k, line += ld, x += S[j]) {
                    const int i1 = static_cast<int>(x >> 32);
                    const float u = frac_of(x);
                    const float p0 = line[i1], p1 = line[i1 + 1];
                    acc = fmaf(u, p1 - p0, acc + p0);
                }
                sum[j] += acc;
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int j = 0; j < kFpMaxRays; ++j) {
        const int r = threadIdx.x + j * kFpThreads;
        if (r < nrays) {
            const int ia = v0 + r / c.ns;
            const double dw = cls[j] == 0 ? fabs(c.dy / sincos[2 * ia + 1]) : fabs(c.dx / sincos[2 * ia]);
            proj[blockIdx.y * c.proj_stride + static_cast<size_t>(v0) * c.ns + r] =
                static_cast<float>(sum[j] * dw);
        }
    }
}

// ---- FP32 forward, row-band pipeline -------------------------------------------
//
// Rays of column-marching views are run on a transposed copy of the image, so
// every ray marches image rows.  A CTA owns kFrViews views x a chunk of
// kFrChunk channels (4 rays of one view per thread, so the view's per-sample
// step S is shared).  The source image streams through shared memory in bands
// of `band` rows: each band is one contiguous range of the row-major image,
// brought in by a single TMA bulk copy (16-byte aligned start, 16-byte multiple
// size; the <= 3 elements of a ragged array tail are loaded directly) into one
// of two buffers, two bands ahead, completing on that buffer's mbarrier.
constexpr int kFrThreads = 256;
constexpr int kFrViews = 4;
constexpr int kFrRaysPerThread = 4;
constexpr int kFrLanesPerView = kFrThreads / kFrViews;          // 64
constexpr int kFrChunk = kFrLanesPerView * kFrRaysPerThread;    // 256 channels

struct FrConst {
    int ns, na, n;          // n = nx = ny
    int band;               // rows per band
    int buf_floats;         // floats per band buffer (>= band*n + 8, multiple of 32)
    long long total;        // elements of one source array (batch * n * n)
    long long total4;       // total rounded down to 4
    double dx, dy;
    size_t proj_stride;
};

__global__ void __launch_bounds__(kFrThreads, 4)
    fp_rows_f32(const float* __restrict__ img, const float* __restrict__ imgT,
                float* __restrict__ proj, const double* __restrict__ sincos,
                const double* __restrict__ bo, const int* __restrict__ usex, const FrConst c)
{
    extern __shared__ __align__(128) unsigned char fr_dyn[];
    float* buf = reinterpret_cast<float*>(fr_dyn + ((128u - (smem_u32(fr_dyn) & 127u)) & 127u));
    __shared__ __align__(8) unsigned long long s_bar[2];
    __shared__ int s_ok;

    const int tid = threadIdx.x;
    const int vl = tid / kFrLanesPerView, lv = tid - vl * kFrLanesPerView;
    const int ia = blockIdx.x * kFrViews + vl;
    const int item = blockIdx.z;
    const bool view_ok = ia < c.na;
    const int cls = view_ok ? (usex[ia] != 0 ? 0 : 1) : -1;

    long long X[kFrRaysPerThread];
    int k0[kFrRaysPerThread], k1[kFrRaysPerThread];
    float sum[kFrRaysPerThread];
    long long S = 0;
#pragma unroll
    for (int j = 0; j < kFrRaysPerThread; ++j) {
        const int is = blockIdx.y * kFrChunk + lv + j * kFrLanesPerView;
        X[j] = 0;
        k0[j] = 0;
        k1[j] = -1;
        sum[j] = 0.0f;
        if (view_ok && is < c.ns) {
            const size_t ray = static_cast<size_t>(ia) * c.ns + is;
            const double begin = bo[2 * ray], step = bo[2 * ray + 1];
            ray_range(begin, step, c.n, c.n - 1, &k0[j], &k1[j]);
            X[j] = ray_line(begin, step, k0[j], k1[j], &S);
        }
    }
    // zero both buffers once: positions never written by a copy then read as 0
    for (int i = tid; i < 2 * c.buf_floats; i += kFrThreads) buf[i] = 0.0f;
    if (tid == 0) {
        mbar_init(smem_u32(&s_bar[0]), 1);
        mbar_init(smem_u32(&s_bar[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int nbands = (c.n + c.band - 1) / c.band;
    unsigned uses0 = 0u, uses1 = 0u;  // completed waits on each barrier (tid 0's count)
    for (int pass = 0; pass < 2; ++pass) {
        if (!__syncthreads_or(cls == pass)) continue;
        const float* src = pass == 0 ? img : imgT;
        const long long item0 = static_cast<long long>(item) * c.n * c.n;
        // band t covers rows [t*band, t*band + nb) = elements [g, g + nb*n) of src
        auto band_start = [&](int t) -> long long {
            return item0 + static_cast<long long>(t) * c.band * c.n;
        };
        auto issue = [&](int t) {
            if (t >= nbands) return;
            const int nb = min(c.band, c.n - t * c.band);
            const long long g = band_start(t), ga = g & ~3ll;
            const long long g1 = min((g + static_cast<long long>(nb) * c.n + 3) & ~3ll, c.total4);
            const unsigned bar = smem_u32(&s_bar[t & 1]);
            const unsigned bytes = g1 > ga ? static_cast<unsigned>((g1 - ga) * sizeof(float)) : 0u;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(bar, bytes);
            if (bytes) bulk_load(smem_u32(buf + (t & 1) * c.buf_floats), src + ga, bytes, bar);
        };
        if (tid == 0) {
            issue(0);
            issue(1);
        }
        for (int t = 0; t < nbands; ++t) {
            const int nb = min(c.band, c.n - t * c.band);
            const long long g = band_start(t), ga = g & ~3ll;
            float* bb = buf + (t & 1) * c.buf_floats;
            if (tid == 0) {
                const unsigned parity = (t & 1) ? (uses1++ & 1u) : (uses0++ & 1u);
                s_ok = mbar_wait_bounded(smem_u32(&s_bar[t & 1]), parity);
                // the ragged tail of the array (not a 16-byte multiple) comes directly
                const long long gend = g + static_cast<long long>(nb) * c.n;
                for (long long i = max(c.total4, ga); i < min(gend, c.total); ++i) bb[i - ga] = src[i];
            }
            __syncthreads();
            if (!s_ok) {
                if (tid == 0) raise_flag(kFlagWaitTimeout);
                return;
            }
            if (cls == pass) {
                const float* base = bb + (g - ga);
                const int b0 = t * c.band;
#pragma unroll
                for (int j = 0; j < kFrRaysPerThread; ++j) {
                    const int ka = max(k0[j], b0), kb = min(k1[j], b0 + nb - 1);
                    if (ka > kb) continue;
                    long long x = X[j] + static_cast<long long>(ka) * S;
                    const float* row = base + (ka - b0) * c.n;
                    float acc = 0.0f;  // this band's partial sum (blocked summation)
#pragma unroll 4
                    for (int k = ka; k <= kb; ++k) {
                        const int i1 = static_cast<int>(x >> 32);
                        const float u = frac_of(x);
                        const float p0 = row[i1], p1 = row[i1 + 1];
                        acc = fmaf(u, p1 - p0, acc + p0);
                        x += S;
                        row += c.n;
                    }
                    sum[j] += acc;
                }
            }
            __syncthreads();
            if (tid == 0) issue(t + 2);
        }
    }
    if (view_ok) {
        const double dw = cls == 0 ? fabs(c.dy / sincos[2 * ia + 1]) : fabs(c.dx / sincos[2 * ia]);
        float* P = proj + item * c.proj_stride + static_cast<size_t>(ia) * c.ns;
#pragma unroll
        for (int j = 0; j < kFrRaysPerThread; ++j) {
            const int is = blockIdx.y * kFrChunk + lv + j * kFrLanesPerView;
            if (is < c.ns) P[is] = static_cast<float>(sum[j] * dw);
        }
    }
}

// imgT[b][x][y] = img[b][y][x] for n x n images (32x32 tiles through shared memory).
__global__ void __launch_bounds__(256) transpose_f32(const float* __restrict__ in, float* __restrict__ out, int n)
{
    __shared__ float t[32][33];
    const size_t off = static_cast<size_t>(blockIdx.z) * n * n;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int y = y0 + r, x = x0 + threadIdx.x;
        if (x < n && y < n) t[r][threadIdx.x] = in[off + static_cast<size_t>(y) * n + x];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int x = x0 + r, y = y0 + threadIdx.x;
        if (x < n && y < n) out[off + static_cast<size_t>(x) * n + y] = t[threadIdx.x][r];
    }
}

// ---- FP32 adjoint: per-pixel gather over each view's channel footprint ----
// Channel positions of pixel centres are 32.32 fixed point built from the
// caller's grad-prep table (one FP64 conversion per tile line and view); the
// footprint and triangle weights are those of src/fp_par_2d.cc:339-383.
constexpr int kFaViews = 16;
constexpr int kFaRows = 4;  // pixels per thread (one column), 32x32 tile

__global__ void __launch_bounds__(256)
    fp_adj_f32(const float* __restrict__ proj, float* __restrict__ img,
               const double* __restrict__ weights, const double* __restrict__ pos,
               const int* __restrict__ usex, const FpConst c)
{
    __shared__ long long s_base[kFaViews][32];
    __shared__ long long s_o1[kFaViews];
    __shared__ float s_w[kFaViews], s_inv[kFaViews];
    __shared__ int s_ux[kFaViews];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tx0 = blockIdx.x * 32, ty0 = blockIdx.y * 32;
    const int ix = tx0 + lane;
    const float* P = proj + blockIdx.z * c.proj_stride;
    float acc[kFaRows];
#pragma unroll
    for (int r = 0; r < kFaRows; ++r) acc[r] = 0.0f;
    const int n = c.nx;  // == ny

    for (int v0 = 0; v0 < c.na; v0 += kFaViews) {
        const int nv = min(kFaViews, c.na - v0);
        for (int idx = threadIdx.x; idx < nv * 32; idx += 256) {
            const int j = idx >> 5, l = idx & 31;
            const int ia = v0 + j;
            const int ux = usex[ia] != 0;
            const int lin = min((ux ? ty0 : tx0) + l, n - 1);
            const double* pp = pos + (static_cast<size_t>(ia) * n + lin) * 2;
            s_base[j][l] = llrint(pp[0] * kTwo32);
            if (l == 0) {
                s_o1[j] = llrint(pp[1] * kTwo32);
                s_w[j] = static_cast<float>(weights[ia]);
                s_inv[j] = static_cast<float>(1.0 / fabs(pp[1]));
                s_ux[j] = ux;
            }
        }
        __syncthreads();
        float blk[kFaRows];  // this view block's partial sums (blocked summation)
#pragma unroll
        for (int r = 0; r < kFaRows; ++r) blk[r] = 0.0f;
        for (int j = 0; j < nv; ++j) {
            const int ux = s_ux[j];
            const long long O1 = s_o1[j];
            const float inv = s_inv[j], w = s_w[j];
            const float* row = P + static_cast<size_t>(v0 + j) * c.ns;
#pragma unroll
            for (int r = 0; r < kFaRows; ++r) {
                const int iy = ty0 + warp * kFaRows + r;
                const int along = ux ? ix : iy;
                const long long MID = s_base[j][ux ? warp * kFaRows + r : lane] +
                                      static_cast<long long>(along) * O1;
                long long L = along == 0 ? MID : MID - O1;
                long long R = along == n - 1 ? MID : MID + O1;
                if (L > R) {
                    const long long t = L;
                    L = R;
                    R = t;
                }
                const int lo = max(static_cast<int>((L + 0xFFFFFFFFll) >> 32), 0);
                const int hi = min(static_cast<int>(R >> 32), c.ns - 1);
                const int mi = static_cast<int>(MID >> 32);
                const float mf = frac_of(MID);
                float part = 0.0f;
                for (int is = lo; is <= hi; ++is) {
                    const float d = fabsf(mf - static_cast<float>(is - mi));
                    part = fmaf(fmaf(-d, inv, 1.0f), __ldg(row + is), part);
                }
                blk[r] = fmaf(part, w, blk[r]);
            }
        }
#pragma unroll
        for (int r = 0; r < kFaRows; ++r) acc[r] += blk[r];
        __syncthreads();
    }
    float* O = img + blockIdx.z * c.img_stride;
#pragma unroll
    for (int r = 0; r < kFaRows; ++r) {
        const int iy = ty0 + warp * kFaRows + r;
        if (ix < c.nx && iy < c.ny) O[static_cast<size_t>(iy) * c.nx + ix] = acc[r];
    }
}

constexpr int kFp64Threads = 128;

template <typename T>
__global__ void __launch_bounds__(kFp64Threads)
    fp_ray_kernel(const T* __restrict__ img, T* __restrict__ proj,
                  const double* __restrict__ sincos, const double* __restrict__ bo,
                  const int* __restrict__ usex, int ns, int na, int nx, int ny, double dx,
                  double dy, size_t img_stride, size_t proj_stride)
{
    const int is = blockIdx.x * kFp64Threads + threadIdx.x;
    const int ia = blockIdx.y;
    if (is >= ns) return;
    const T* I = img + blockIdx.z * img_stride;
    const size_t ray = static_cast<size_t>(ia) * ns + is;
    const bool ux = usex[ia] != 0;
    const double begin = bo[2 * ray], step = bo[2 * ray + 1];
    const int nsamp = ux ? ny : nx;
    const int lim = ux ? nx - 1 : ny - 1;
    T sum = 0;
    {
        double x = begin;
        for (int k = 0; k < nsamp; ++k) {
            if (x >= 0 && x <= lim) {
                const int i1 = static_cast<int>(floor(x));
                const int i2 = static_cast<int>(ceil(x));
                const double u = x - i1;
                if (ux)
                    sum += (1 - u) * I[i1 + static_cast<size_t>(k) * nx] + u * I[i2 + static_cast<size_t>(k) * nx];
                else
                    sum += (1 - u) * I[k + static_cast<size_t>(i1) * nx] + u * I[k + static_cast<size_t>(i2) * nx];
            }
            x += step;
        }
    }
    const double dw = ux ? fabs(dy / sincos[2 * ia + 1]) : fabs(dx / sincos[2 * ia]);
    proj[blockIdx.z * proj_stride + ray] = static_cast<T>(sum * static_cast<T>(dw));
}

template <typename T>
__global__ void fp_adj_kernel(const T* __restrict__ proj, T* __restrict__ img,
                              const double* __restrict__ weights, const double* __restrict__ pos,
                              const int* __restrict__ usex, int ns, int na, int nx, int ny,
                              size_t proj_stride, size_t img_stride)
{
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * 8 + threadIdx.y;
    if (ix >= nx || iy >= ny) return;
    const T* P = proj + blockIdx.z * proj_stride;
    double sum = 0.0;
    for (int ia = 0; ia < na; ++ia) {
        const bool ux = usex[ia] != 0;
        const double* pp = pos + static_cast<size_t>(ia) * 2 * nx;
        const int lin = ux ? iy : ix;   // table entry
        const int along = ux ? ix : iy; // position along the entry
        const int last = ux ? nx - 1 : ny - 1;
        T begin, step;
        begin = static_cast<T>(pp[2 * lin]);
        step = static_cast<T>(pp[2 * lin + 1]);
        const T mid = begin + step * static_cast<T>(along);
        T left = along == 0 ? mid : mid - step;
        T right = along == last ? mid : mid + step;
        if (left > right) {
            const T t = left;
            left = right;
            right = t;
        }
        T lo = ceil(left), hi = floor(right);
        if (lo < 0) lo = 0;
        if (hi > static_cast<T>(ns - 1)) hi = static_cast<T>(ns - 1);
        const T* row = P + static_cast<size_t>(ia) * ns;
        const T inv = static_cast<T>(1) / step;
        T part = 0;
        for (int is = static_cast<int>(lo); is <= static_cast<int>(hi); ++is) {
            const T t = (mid - static_cast<T>(is)) * inv;
            part += (static_cast<T>(1) - (t < 0 ? -t : t)) * row[is];
        }
        sum += static_cast<double>(part) * weights[ia];
    }
    img[blockIdx.z * img_stride + static_cast<size_t>(iy) * nx + ix] = static_cast<T>(sum);
}

int check_fp(const ctr_par_param* p, const void* a, const void* b, const void* t0,
             const void* t1, const void* t2, int batch)
{
    if (!p || !a || !b || !t0 || !t1 || !t2) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (p->ns < 1 || p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (p->nx != p->ny) return fail(CTR_ERR_INVALID_ARG, "ray-driven projection needs nx == ny");
    if (batch > 65535 || p->na > 65535) return fail(CTR_ERR_UNSUPPORTED, "batch or na > 65535");
    return CTR_OK;
}

FpConst fp_const(const ctr_par_param* p)
{
    FpConst c{};
    c.ns = p->ns; c.na = p->na; c.nx = p->nx; c.ny = p->ny;
    c.dx = p->dx; c.dy = p->dy;
    c.img_stride = static_cast<size_t>(p->nx) * p->ny;
    c.proj_stride = static_cast<size_t>(p->ns) * p->na;
    return c;
}

template <typename T>
int fp_forward(const ctr_par_param* p, const T* img, T* proj, const double* sc,
               const double* bo, const int* usex, int batch, cudaStream_t stream)
{
    int st = check_fp(p, img, proj, sc, bo, usex, batch);
    if (st) return st;
    if constexpr (sizeof(T) == 4) {
        const int n = static_cast<int>(p->nx);
        FrConst r{};
        r.ns = p->ns; r.na = p->na; r.n = n;
        r.band = std::max(2, std::min(32, 4096 / n));
        r.buf_floats = (r.band * n + 8 + 31) / 32 * 32;
        r.total = static_cast<long long>(batch) * n * n;
        r.total4 = r.total & ~3ll;
        r.dx = p->dx; r.dy = p->dy;
        r.proj_stride = static_cast<size_t>(p->ns) * p->na;
        const size_t smem = 128 + 2 * static_cast<size_t>(r.buf_floats) * sizeof(float);
        if (smem <= 160 * 1024 && reinterpret_cast<uintptr_t>(img) % 16 == 0 && r.total < (1ll << 40)) {
            // column-marching views run on the transposed image (stream-ordered scratch)
            float* imgT = nullptr;
            cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&imgT), r.total * sizeof(float), stream);
            if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d scratch: %s", cudaGetErrorString(e));
            transpose_f32<<<dim3(div_up(n, 32), div_up(n, 32), batch), dim3(32, 8), 0, stream>>>(img, imgT, n);
            int st2 = check_launch("fp_par_2d transpose");
            if (st2 == CTR_OK) {
                e = cudaFuncSetAttribute(fp_rows_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
                if (e != cudaSuccess) {
                    st2 = fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
                } else {
                    dim3 grid(div_up(p->na, kFrViews), div_up(p->ns, kFrChunk), batch);
                    fp_rows_f32<<<grid, kFrThreads, smem, stream>>>(img, imgT, proj, sc, bo, usex, r);
                    st2 = check_launch("fp_par_2d");
                }
            }
            cudaFreeAsync(imgT, stream);
            return st2;
        }
        // fallback: image bands staged with plain loads
        FpConst c = fp_const(p);
        c.views = std::max(1, std::min(4, kFpThreads * kFpMaxRays / static_cast<int>(p->ns)));
        if (c.views * static_cast<long long>(p->ns) > kFpThreads * kFpMaxRays)
            return fail(CTR_ERR_UNSUPPORTED, "fp_par_2d: ns=%u exceeds %d channels", p->ns,
                        kFpThreads * kFpMaxRays);
        const int len = std::max(p->nx, p->ny) + 1;
        c.band = std::max(1, std::min(32, 16384 / len));
        const size_t smem2 = sizeof(float) * static_cast<size_t>(c.band) * len;
        cudaError_t e = cudaFuncSetAttribute(fp_band_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem2));
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
        dim3 grid(div_up(p->na, c.views), batch);
        fp_band_f32<<<grid, kFpThreads, smem2, stream>>>(img, proj, sc, bo, usex, c);
    } else {
        dim3 grid(div_up(p->ns, kFp64Threads), p->na, batch);
        fp_ray_kernel<T><<<grid, kFp64Threads, 0, stream>>>(img, proj, sc, bo, usex, p->ns, p->na,
                                                            p->nx, p->ny, p->dx, p->dy,
                                                            static_cast<size_t>(p->nx) * p->ny,
                                                            static_cast<size_t>(p->ns) * p->na);
    }
    return check_launch("fp_par_2d");
}

template <typename T>
int fp_adjoint(const ctr_par_param* p, const T* proj, T* img, const double* w,
               const double* pos, const int* usex, int batch, cudaStream_t stream)
{
    int st = check_fp(p, proj, img, w, pos, usex, batch);
    if (st) return st;
    if constexpr (sizeof(T) == 4) {
        FpConst c = fp_const(p);
        dim3 grid(div_up(p->nx, 32), div_up(p->ny, 32), batch);
        fp_adj_f32<<<grid, 256, 0, stream>>>(proj, img, w, pos, usex, c);
    } else {
        dim3 grid(div_up(p->nx, 32), div_up(p->ny, 8), batch);
        fp_adj_kernel<T><<<grid, dim3(32, 8), 0, stream>>>(proj, img, w, pos, usex, p->ns, p->na,
                                                           p->nx, p->ny,
                                                           static_cast<size_t>(p->ns) * p->na,
                                                           static_cast<size_t>(p->nx) * p->ny);
    }
    return check_launch("fp_par_2d_grad");
}

// ---- allocation-free FP32 forward projection ---------------------------------
// For callers that must not allocate device memory inside a call: a host
// framework that hands out all device memory itself (its own pool, a fixed
// arena), or a real-time loop that cannot wait on the allocator.  The
// transposed image that column-marching views read lives in this fixed
// file-scope array instead of stream-ordered scratch: at most
// kFpNoAllocFloats = 4,194,304 floats (16 MiB), i.e. batch * nx * ny <= 2^22
// (one 2048^2 image, or 16 images of 512^2).  The transpose overwrites every
// element it later reads, so nothing in the array has to start at zero.
// All calls on a device share the one array: calls ordered on one stream are
// safe, calls that can overlap (two streams, two host threads without
// ordering) race on it and give wrong results.
constexpr long long kFpNoAllocFloats = 1ll << 22;
static __device__ __align__(256) float g_fp_noalloc_scratch[kFpNoAllocFloats];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
float* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// The array's device address on the current device, looked up once per device
// (cudaGetSymbolAddress; the first call on a device does this set-up).
int noalloc_scratch(float** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(CTR_ERR_DEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(CTR_ERR_UNSUPPORTED, "device %d >= %d", dev, kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_fp_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(CTR_ERR_CUDA, "fp_par_2d_f32_noalloc scratch address: %s",
                        cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<float*>(ptr);
    }
    *out = g_noalloc_ptr[dev];
    return CTR_OK;
}

int fp_forward_noalloc(const ctr_par_param* p, const float* img, float* proj, const double* sc,
                       const double* bo, const int* usex, int batch, cudaStream_t stream)
{
    int st = check_fp(p, img, proj, sc, bo, usex, batch);
    if (st) return st;
    const long long n = p->nx;
    if (n > 2048 || batch * n * n > kFpNoAllocFloats)
        return fail(CTR_ERR_UNSUPPORTED,
                    "fp_par_2d_f32_noalloc: batch*nx*ny = %d*%lld*%lld exceeds its fixed scratch of "
                    "%lld floats (16 MiB); split the batch or call ctr_fp_par_2d_f32",
                    batch, n, n, kFpNoAllocFloats);
    if (reinterpret_cast<uintptr_t>(img) % 16 != 0)
        return fail(CTR_ERR_INVALID_ARG, "fp_par_2d_f32_noalloc: img must be 16-byte aligned");
    FrConst r{};
    r.ns = p->ns; r.na = p->na; r.n = static_cast<int>(n);
    r.band = std::max(2, std::min(32, static_cast<int>(4096 / n)));
    r.buf_floats = (r.band * r.n + 8 + 31) / 32 * 32;
    r.total = batch * n * n;
    r.total4 = r.total & ~3ll;
    r.dx = p->dx; r.dy = p->dy;
    r.proj_stride = static_cast<size_t>(p->ns) * p->na;
    const size_t smem = 128 + 2 * static_cast<size_t>(r.buf_floats) * sizeof(float);
    float* imgT = nullptr;
    st = noalloc_scratch(&imgT);
    if (st) return st;
    transpose_f32<<<dim3(div_up(n, 32), div_up(n, 32), batch), dim3(32, 8), 0, stream>>>(
        img, imgT, r.n);
    st = check_launch("fp_par_2d_f32_noalloc transpose");
    if (st) return st;
    cudaError_t e = cudaFuncSetAttribute(fp_rows_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
    dim3 grid(div_up(p->na, kFrViews), div_up(p->ns, kFrChunk), batch);
    fp_rows_f32<<<grid, kFrThreads, smem, stream>>>(img, imgT, proj, sc, bo, usex, r);
    return check_launch("fp_par_2d_f32_noalloc");
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_fp_par_2d_f32(const ctr_par_param* p, const float* img, float* proj,
                      const double* sincostbl, const double* beginoffset, const int* usex,
                      int batch, cudaStream_t stream)
{
    return fp_forward<float>(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}
int ctr_fp_par_2d_f64(const ctr_par_param* p, const double* img, double* proj,
                      const double* sincostbl, const double* beginoffset, const int* usex,
                      int batch, cudaStream_t stream)
{
    return fp_forward<double>(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}
int ctr_fp_par_2d_grad_f32(const ctr_par_param* p, const float* proj, float* img,
                           const double* weights, const double* pos, const int* usex,
                           int batch, cudaStream_t stream)
{
    return fp_adjoint<float>(p, proj, img, weights, pos, usex, batch, stream);
}
int ctr_fp_par_2d_grad_f64(const ctr_par_param* p, const double* proj, double* img,
                           const double* weights, const double* pos, const int* usex,
                           int batch, cudaStream_t stream)
{
    return fp_adjoint<double>(p, proj, img, weights, pos, usex, batch, stream);
}
int ctr_fp_par_2d_f32_noalloc(const ctr_par_param* p, const float* img, float* proj,
                              const double* sincostbl, const double* beginoffset, const int* usex,
                              int batch, cudaStream_t stream)
{
    return fp_forward_noalloc(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}

}  // extern "C"
