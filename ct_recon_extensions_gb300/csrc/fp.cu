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

#include "ctr_common.cuh"

namespace ctr {
namespace {

// ---- FP32 forward: image bands in shared memory, fixed-point sample positions

constexpr int kFpThreads = 512;
constexpr int kFpMaxRays = 8;  // rays per thread
// Sample positions are 32.32 fixed point.  Rounding the per-ray start and step
// to 2^-32 moves a position by at most (k+1)/2 units (< 1100 units for 2048
// samples); the bias keeps X >= 0 wherever the FP64 position is >= 0, so the
// integer part is a valid pixel index (it shifts positions by 4.8e-7 px).
constexpr long long kFpBias = 2048;
constexpr double kTwo32 = 4294967296.0;

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
            X[j] = llrint(begin * kTwo32) + kFpBias;
            S[j] = llrint(step * kTwo32);
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
                float acc = sum[j];
                for (int k = ka; k <= kb; ++k, line += ld, x += S[j]) {
                    const int i1 = static_cast<int>(x >> 32);
                    const float u = frac_of(x);
                    const float p0 = line[i1], p1 = line[i1 + 1];
                    acc = fmaf(u, p1 - p0, acc + p0);
                }
                sum[j] = acc;
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
                acc[r] = fmaf(part, w, acc[r]);
            }
        }
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
        FpConst c = fp_const(p);
        c.views = std::max(1, std::min(4, kFpThreads * kFpMaxRays / static_cast<int>(p->ns)));
        if (c.views * static_cast<long long>(p->ns) > kFpThreads * kFpMaxRays)
            return fail(CTR_ERR_UNSUPPORTED, "fp_par_2d: ns=%u exceeds %d channels", p->ns,
                        kFpThreads * kFpMaxRays);
        const int len = std::max(p->nx, p->ny) + 1;
        c.band = std::max(1, std::min(32, 16384 / len));
        const size_t smem = sizeof(float) * static_cast<size_t>(c.band) * len;
        cudaError_t e = cudaFuncSetAttribute(fp_band_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
        dim3 grid(div_up(p->na, c.views), batch);
        fp_band_f32<<<grid, kFpThreads, smem, stream>>>(img, proj, sc, bo, usex, c);
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

}  // extern "C"
