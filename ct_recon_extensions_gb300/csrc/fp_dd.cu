// Distance-driven parallel forward projection and the reference's
// distance-driven gradient (src/fp_par_2d.cc:396-653).
//
// Forward: a ray's footprint on each line of the marched axis is [left,
// right] (running FP64 sums from the channel's centre +- half width).  It
// averages the trapezoid (p[i] + p[i+1]) / 2 of neighbouring pixels over the
// pixel intervals [i, i+1] it covers, weighted by the covered length, and the
// line adds tsum / lsum.  The reference's pixel loop runs an unsigned index
// from floor(left): a negative floor converts (undefined in C++) to a huge
// value on the x86-64 build that its fixtures come from, so such a line adds
// nothing; intervals from nx-1 on are skipped.  Positions, the line's
// interval range and the two partial lengths (first and last interval) are
// FP64 as in the reference, so every decision is the reference's; for
// T = float the sums run in FP32 as the reference's T sums do.  One thread per
// ray.
//
// Grad (the reference's, not the adjoint of the normalised forward): per
// pixel and view the channel footprint around the pixel's channel mid (mid -
// offset .. mid + offset, one-sided at the image edges) gathers
// length * proj / 2 over channels ceil(left - 0.5) .. floor(right + 0.5); a
// negative first channel skips the view (the same unsigned index), and
// channels past ns read on into the next view's row as the reference's
// unchecked index does (0 past the last view).  One thread per pixel.
#include <cmath>
#include <type_traits>
#include <vector>

#include "ctr_common.cuh"
#include "fp_setup.cuh"

namespace ctr {
namespace {

constexpr int kDdThreads = 128;
constexpr double kDdPi = 3.14159265358979323846;

// Fraction of a 32.32 fixed-point value, from its low word's top 23 bits.
__device__ __forceinline__ float dd_frac(long long X)
{
    return __uint_as_float(0x3F800000u | (static_cast<unsigned>(X) >> 9)) - 1.0f;
}

// imgT[b][x][y] = img[b][y][x] (32 x 32 tiles)
__global__ void __launch_bounds__(256) dd_transpose(const float* __restrict__ img, float* __restrict__ imgT, int n)
{
    __shared__ float t[32][33];
    const size_t off = static_cast<size_t>(blockIdx.z) * n * n;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8)
        if (x0 + tx < n && y0 + r < n) t[r][tx] = img[off + static_cast<size_t>(y0 + r) * n + x0 + tx];
    __syncthreads();
    for (int r = ty; r < 32; r += 8)
        if (y0 + tx < n && x0 + r < n) imgT[off + static_cast<size_t>(x0 + r) * n + y0 + tx] = t[tx][r];
}

// One ray of the forward with the reference's own arithmetic: FP64 edges,
// interval range and lengths; sums in T (FP32 for T = float).
template <typename T>
__device__ T dd_ray_exact(const T* __restrict__ I, const double* __restrict__ b, int ux, int nl, int nal,
                          int nx)
{
    const size_t step_line = ux ? static_cast<size_t>(nx) : 1;   // next line
    const size_t step_pix = ux ? 1 : static_cast<size_t>(nx);    // next pixel along the line
    const double off = b[1];
    double left = __dsub_rn(b[0], b[2]), right = __dadd_rn(b[0], b[2]);
    if (left > right) {
        const double t = left;
        left = right;
        right = t;
    }
    T sum = 0;
    for (int l = 0; l < nl; ++l) {
        const double fl = floor(left), cr = ceil(right);
        T tsum = 0, lsum = 0;
        if (fl >= 0.0) {
            // intervals i0 .. (i < cr), all but those from nal - 1 on
            const int i0 = static_cast<int>(fl);
            const int iend = cr < static_cast<double>(nal - 1) ? static_cast<int>(cr) : nal - 1;
            const T* line = I + static_cast<size_t>(l) * step_line;
            for (int i = i0; i < iend; ++i) {
                const double a = static_cast<double>(i + 1) < right ? static_cast<double>(i + 1) : right;
                const double c = static_cast<double>(i) > left ? static_cast<double>(i) : left;
                const double len = a - c;
                const T p0 = line[static_cast<size_t>(i) * step_pix];
                const T p1 = line[static_cast<size_t>(i + 1) * step_pix];
                if constexpr (sizeof(T) == 4) {
                    const float lf = static_cast<float>(len);
                    tsum = fmaf(lf, (p0 + p1) * 0.5f, tsum);
                    lsum += lf;
                } else {
                    tsum += len * (p0 + p1) / 2;
                    lsum += len;
                }
            }
        }
        if (lsum > 0) sum += tsum / lsum;
        left += off;
        right += off;
    }
    return sum;
}

// FP64 forward: the reference's loop, one thread per ray.
__global__ void __launch_bounds__(kDdThreads)
    fp_dd_f64(const double* __restrict__ img, double* __restrict__ proj, const double* __restrict__ sincos,
              const double* __restrict__ bo, const int* __restrict__ usex, int ns, int na, int nx, int ny,
              double dx, double dy, size_t img_stride, size_t proj_stride)
{
    const long long ray = static_cast<long long>(blockIdx.x) * kDdThreads + threadIdx.x;
    if (ray >= static_cast<long long>(na) * ns) return;
    const int ia = static_cast<int>(ray / ns);
    const int ux = usex[ia];
    const double w = ux ? fabs(dy / sincos[2 * ia + 1]) : fabs(dx / sincos[2 * ia]);
    const double sum = dd_ray_exact<double>(img + blockIdx.y * img_stride, bo + 3 * ray, ux, ux ? ny : nx,
                                            ux ? nx : ny, nx);
    proj[blockIdx.y * proj_stride + ray] = sum * w;
}

// FP32 forward.  The reference's discontinuous decisions come down to which
// lines count: a line adds tsum / lsum iff its footprint start satisfies
// 0 <= left < n-1 (a negative start skips it; from n-1 on no interval is
// left), a contiguous range of lines since left is a running sum.  That range
// is decided as the reference decides it (axis_range, and a line exactly at
// n-1 dropped after an exact check).  Inside it both edges march in 32.32
// fixed point, and the covered lengths are FP32 relative to the first
// interval; everything else varies continuously with the edges.  Lines of
// column-marching views read the transposed copy, so a warp's loads stay
// within a few rows.  Rays outside the fixed-point range take dd_ray_exact.
__global__ void __launch_bounds__(kDdThreads)
    fp_dd_f32(const float* __restrict__ img, const float* __restrict__ imgT, float* __restrict__ proj,
              const double* __restrict__ sincos, const double* __restrict__ bo, const int* __restrict__ usex,
              int ns, int na, int n, double dx, double dy, size_t img_stride, size_t proj_stride)
{
    const long long ray = static_cast<long long>(blockIdx.x) * kDdThreads + threadIdx.x;
    if (ray >= static_cast<long long>(na) * ns) return;
    const int ia = static_cast<int>(ray / ns);
    const int ux = usex[ia];
    const float w = static_cast<float>(ux ? fabs(dy / sincos[2 * ia + 1]) : fabs(dx / sincos[2 * ia]));
    const double* b = bo + 3 * ray;
    float* out = proj + blockIdx.y * proj_stride + ray;
    const double off = b[1];
    double left0 = __dsub_rn(b[0], b[2]), right0 = __dadd_rn(b[0], b[2]);
    if (left0 > right0) {
        const double t = left0;
        left0 = right0;
        right0 = t;
    }
    const int er = static_cast<int>((double_bits(right0) >> 52) & 0x7FF);
    const int el = static_cast<int>((double_bits(left0) >> 52) & 0x7FF);
    const int eo = static_cast<int>((double_bits(off) >> 52) & 0x7FF);
    if (er >= 1043 || el >= 1043 || eo >= 1025 || n < 2) {  // beyond the fixed-point range
        *out = dd_ray_exact<float>(img + blockIdx.y * img_stride, b, ux, n, n, n) * w;
        return;
    }
    long long XL, S;
    int k0, k1;
    axis_range(left0, off, n, n, &XL, &S, &k0, &k1);
    // a start exactly at n-1 leaves no interval: the range's end there drops
    if (k0 <= k1) {
        const double lim = static_cast<double>(n - 1);
        const long long L = static_cast<long long>(n - 1) << 32, T = tie_units(n);
        if (off == 0.0) {
            if (left0 == lim) k1 = k0 - 1;
        } else {
            const int ke = off > 0.0 ? k1 : k0;
            const long long X = XL + static_cast<long long>(ke) * S;
            if (X > L - T && X < L + T) {
                AccWalk wk{left0, 0};
                acc_advance(&wk, off, ke);
                if (wk.x == lim) {
                    if (off > 0.0) --k1;
                    else ++k0;
                }
            }
        }
    }
    const float* I = (ux ? img : imgT) + blockIdx.y * img_stride;  // lines are rows of I
    const long long XR = fix32(right0) + (XL - fix32(left0));        // the same anchor as the left edge
    long long xl = XL + static_cast<long long>(k0) * S, xr = XR + static_cast<long long>(k0) * S;
    float sum = 0.0f;
    for (int l = k0; l <= k1; ++l) {
        const int h = static_cast<int>(xl >> 32);
        const int i0 = min(max(h, 0), n - 2);
        // the start relative to interval i0 (clamped: the fixed-point start may
        // sit a hair outside [0, n-1) where the exact one is inside)
        const float lr = h == i0 ? dd_frac(xl) : (h < 0 ? 0.0f : 1.0f);
        const int hr = static_cast<int>(xr >> 32);
        const float rr = static_cast<float>(hr - i0) + dd_frac(xr);
        const int ie = min(hr + (static_cast<unsigned>(xr) != 0u ? 1 : 0), n - 1);
        const float* line = I + static_cast<size_t>(l) * n;
        float tsum = 0.0f, lsum = 0.0f;
        for (int i = i0; i < ie; ++i) {
            const float j = static_cast<float>(i - i0);
            const float len = fmaxf(fminf(j + 1.0f, rr) - fmaxf(j, lr), 0.0f);
            tsum = fmaf(len, (__ldg(line + i) + __ldg(line + i + 1)) * 0.5f, tsum);
            lsum += len;
        }
        // a counted line always covers part of interval i0; where the clamped
        // fixed-point edges leave no length, that sliver's trapezoid is the mean
        sum += lsum > 0.0f ? tsum / lsum : (__ldg(line + i0) + __ldg(line + i0 + 1)) * 0.5f;
        xl += S;
        xr += S;
    }
    *out = sum * w;
}

// The reference's distance-driven grad in FP64 (T = double), one thread per
// pixel: edges, channel range, lengths and sums with its operations.
template <typename T>
__global__ void __launch_bounds__(kDdThreads)
    fp_dd_grad_kernel(const T* __restrict__ proj, T* __restrict__ img, const double* __restrict__ weights,
                      const double* __restrict__ pos, const int* __restrict__ usex, int ns, int na, int nx,
                      int ny, size_t img_stride, size_t proj_stride)
{
    const long long pix = static_cast<long long>(blockIdx.x) * kDdThreads + threadIdx.x;
    if (pix >= static_cast<long long>(nx) * ny) return;
    const int iy = static_cast<int>(pix / nx), ix = static_cast<int>(pix - static_cast<long long>(iy) * nx);
    const T* P = proj + blockIdx.y * proj_stride;
    const size_t total = static_cast<size_t>(na) * ns;
    static_assert(sizeof(T) == 8, "the FP32 grad is fp_dd_grad_f32");
    T sum = 0;
    for (int ia = 0; ia < na; ++ia) {
        const double* pp = pos + static_cast<size_t>(ia) * nx * 2;
        double mid, left, right;
        if (usex[ia]) {
            const double begin = pp[2 * iy], off = pp[2 * iy + 1];
            mid = __dadd_rn(begin, __dmul_rn(off, static_cast<double>(ix)));
            left = ix == 0 ? mid : __dsub_rn(mid, off);
            right = ix == nx - 1 ? mid : __dadd_rn(mid, off);
        } else {
            const double begin = pp[2 * ix], off = pp[2 * ix + 1];
            mid = __dadd_rn(begin, __dmul_rn(off, static_cast<double>(iy)));
            left = iy == 0 ? mid : __dsub_rn(mid, off);
            right = iy == ny - 1 ? mid : __dadd_rn(mid, off);
        }
        if (left > right) {
            const double t = left;
            left = right;
            right = t;
        }
        const double c0 = ceil(__dsub_rn(left, 0.5)), c1 = floor(__dadd_rn(right, 0.5));
        if (!(c0 >= 0.0)) continue;
        // channels past the sinogram's end add 0: the loop stops there (finite
        // for any input)
        const double last = fmin(c1, static_cast<double>(total - 1 - static_cast<size_t>(ia) * ns));
        const int first = static_cast<int>(fmin(c0, last + 1.0));
        T tmp = 0;
        for (int is = first; static_cast<double>(is) <= last; ++is) {
            const double hi = __dadd_rn(static_cast<double>(is), 0.5), lo = __dsub_rn(static_cast<double>(is), 0.5);
            const double len = __dsub_rn(hi < right ? hi : right, lo > left ? lo : left);
            tmp += len * P[static_cast<size_t>(ia) * ns + is] / 2;
        }
        sum += tmp * weights[ia];
    }
    img[blockIdx.y * img_stride + pix] = static_cast<T>(sum);
}

// ---- FP32 grad with fixed-point decisions ---------------------------------------
// Per (pixel, view) the grad's only discontinuous decisions are
// c0 = ceil(left - 0.5) (the view counts iff c0 >= 0; its first channel) and
// c1 = floor(right + 0.5) (its last channel), left/right = begin + off*k -/+ off
// from the reference's FP64 (view, line) table.  A per-call prologue turns that
// table into 32.32 fixed point; the edges are then exact integer arithmetic
// within (1 + (k+1)/2) * 2^-32 of the exact values, and the reference's FP64
// edges are within 1e-12 of those.  Wherever left - 0.5 or right + 0.5 lies
// within kDdFxGuard (2^-16) of an integer the pair reruns the FP64 decision
// code, so every decision is the reference's.  Overlap lengths come from the
// fixed-point offsets to the first channel, in FP32.
struct DdGradFx {
    long long b, o;  // begin and step of one (view, line), 32.32 fixed point; b == kDdFxBad: use FP64
};
constexpr long long kDdFxBad = -0x7fffffffffffffffLL - 1;
constexpr long long kDdHalf = 1LL << 31;
constexpr unsigned kDdFxGuard = 1u << 16;

__global__ void dd_grad_fx_prep(const double* __restrict__ pos, const double* __restrict__ weights,
                                DdGradFx* __restrict__ fx, float* __restrict__ wf, int na, int nx)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < na) wf[i] = static_cast<float>(weights[i]);
    if (i >= static_cast<long long>(na) * nx) return;
    const double b = pos[2 * i], o = pos[2 * i + 1];
    DdGradFx e{kDdFxBad, 0};
    // |begin|, |off| * nx and the edges stay far inside the 64-bit range
    if (fabs(b) < 1073741824.0 && fabs(o) * (nx + 1) < 1073741824.0)
        e = DdGradFx{__double2ll_rn(b * 4294967296.0), __double2ll_rn(o * 4294967296.0)};
    fx[i] = e;
}

// The reference's FP64 decisions for one (pixel, view): false when the view
// adds nothing; else the first channel, the channel count and the edges
// relative to the first channel.
__device__ __forceinline__ bool dd_grad_decide64(const double* __restrict__ pp, int ux, int ix, int iy, int nx,
                                                 int ny, long long room, int& first, int& cnt, float& lr,
                                                 float& rr)
{
    double mid, left, right;
    if (ux) {
        const double begin = pp[2 * iy], off = pp[2 * iy + 1];
        mid = __dadd_rn(begin, __dmul_rn(off, static_cast<double>(ix)));
        left = ix == 0 ? mid : __dsub_rn(mid, off);
        right = ix == nx - 1 ? mid : __dadd_rn(mid, off);
    } else {
        const double begin = pp[2 * ix], off = pp[2 * ix + 1];
        mid = __dadd_rn(begin, __dmul_rn(off, static_cast<double>(iy)));
        left = iy == 0 ? mid : __dsub_rn(mid, off);
        right = iy == ny - 1 ? mid : __dadd_rn(mid, off);
    }
    if (left > right) {
        const double t = left;
        left = right;
        right = t;
    }
    const double c0 = ceil(__dsub_rn(left, 0.5)), c1 = floor(__dadd_rn(right, 0.5));
    if (!(c0 >= 0.0)) return false;
    const double last = fmin(c1, static_cast<double>(room));
    first = static_cast<int>(fmin(c0, last + 1.0));
    cnt = static_cast<int>(last) - first + 1;
    lr = static_cast<float>(__dsub_rn(left, static_cast<double>(first)));
    rr = static_cast<float>(__dsub_rn(right, static_cast<double>(first)));
    return true;
}

__global__ void __launch_bounds__(kDdThreads)
    fp_dd_grad_f32(const float* __restrict__ proj, float* __restrict__ img, const double* __restrict__ pos,
                   const DdGradFx* __restrict__ fx, const float* __restrict__ wf, const int* __restrict__ usex,
                   int ns, int na, int nx, int ny, size_t img_stride, size_t proj_stride)
{
    const long long pix = static_cast<long long>(blockIdx.x) * kDdThreads + threadIdx.x;
    if (pix >= static_cast<long long>(nx) * ny) return;
    const int iy = static_cast<int>(pix / nx), ix = static_cast<int>(pix - static_cast<long long>(iy) * nx);
    const float* P = proj + blockIdx.y * proj_stride;
    const long long total = static_cast<long long>(na) * ns;
    float sum = 0.0f;
    for (int ia = 0; ia < na; ++ia) {
        const int ux = usex[ia];
        const int line = ux ? iy : ix, k = ux ? ix : iy, kmax = ux ? nx - 1 : ny - 1;
        // channels past the sinogram's end add 0: the loop stops there
        const long long room = total - 1 - static_cast<long long>(ia) * ns;
        const DdGradFx e = fx[static_cast<size_t>(ia) * nx + line];
        int first = 0, cnt = 0;
        float lr = 0.0f, rr = 0.0f;
        bool exact = e.b == kDdFxBad;
        if (!exact) {
            const long long mid = e.b + e.o * k;
            long long left = k == 0 ? mid : mid - e.o, right = k == kmax ? mid : mid + e.o;
            if (left > right) {
                const long long t = left;
                left = right;
                right = t;
            }
            const long long L = left - kDdHalf, R = right + kDdHalf;
            const unsigned lf = static_cast<unsigned>(L), rf = static_cast<unsigned>(R);
            if (lf < kDdFxGuard || lf > 0u - kDdFxGuard || rf < kDdFxGuard || rf > 0u - kDdFxGuard) {
                exact = true;  // an edge within 2^-16 of a decision boundary
            } else {
                const long long c0 = (L >> 32) + 1;  // ceil: the fraction is nonzero here
                const long long c1 = R >> 32;         // floor
                if (c0 < 0) continue;
                const long long last = c1 < room ? c1 : room;
                const long long f = c0 < last + 1 ? c0 : last + 1;
                const long long dl = left - (f << 32), dr = right - (f << 32);
                if (dl <= -(1LL << 38) || dl >= (1LL << 38) || dr <= -(1LL << 38) || dr >= (1LL << 38)) {
                    exact = true;  // a footprint wider than the FP32 offsets' range
                } else {
                    first = static_cast<int>(f);
                    cnt = static_cast<int>(last - f + 1);
                    lr = static_cast<float>(static_cast<int>(dl >> 8)) * 5.9604644775390625e-8f;  // 2^-24
                    rr = static_cast<float>(static_cast<int>(dr >> 8)) * 5.9604644775390625e-8f;
                }
            }
        }
        if (exact && !dd_grad_decide64(pos + static_cast<size_t>(ia) * nx * 2, ux, ix, iy, nx, ny, room, first,
                                       cnt, lr, rr))
            continue;
        const float* row = P + static_cast<size_t>(ia) * ns + first;
        float tmp = 0.0f;
        for (int j = 0; j < cnt; ++j) {
            const float fj = static_cast<float>(j);
            const float len = fminf(fj + 0.5f, rr) - fmaxf(fj - 0.5f, lr);
            tmp = fmaf(len, __ldg(row + j) * 0.5f, tmp);
        }
        sum = fmaf(tmp, wf[ia], sum);
    }
    img[blockIdx.y * img_stride + pix] = sum;
}

int check_dd(const ctr_par_param* p, const void* a, const void* b, const void* t0, const void* t1,
             const void* t2, int batch)
{
    if (!p || bad_ptr(a) || bad_ptr(b) || bad_ptr(t0) || bad_ptr(t1) || bad_ptr(t2))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (p->ns < 1 || p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (p->nx != p->ny) return fail(CTR_ERR_INVALID_ARG, "distance-driven projection needs nx == ny");
    if (batch > 65535) return fail(CTR_ERR_UNSUPPORTED, "batch > 65535");
    if (a == b) return fail(CTR_ERR_INVALID_ARG, "projection cannot run in place");
    return CTR_OK;
}

template <typename T>
int dd_forward(const ctr_par_param* p, const T* img, T* proj, const double* sc, const double* bo, const int* usex,
               int batch, cudaStream_t stream)
{
    int st = check_dd(p, img, proj, sc, bo, usex, batch);
    if (st) return st;
    const unsigned long long rays = static_cast<unsigned long long>(p->na) * p->ns;
    const size_t is = static_cast<size_t>(p->nx) * p->ny, ps = static_cast<size_t>(p->na) * p->ns;
    const dim3 grid(div_up(rays, kDdThreads), batch);
    if constexpr (sizeof(T) == 8) {
        fp_dd_f64<<<grid, kDdThreads, 0, stream>>>(img, proj, sc, bo, usex, p->ns, p->na, p->nx, p->ny, p->dx,
                                                   p->dy, is, ps);
        return check_launch("fp_par_2d distance driven");
    } else {
        const int n = static_cast<int>(p->nx);
        if (batch > 65535) return fail(CTR_ERR_UNSUPPORTED, "batch > 65535");
        float* imgT = nullptr;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&imgT), sizeof(float) * is * batch, stream);
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "distance-driven scratch: %s", cudaGetErrorString(e));
        dd_transpose<<<dim3(div_up(n, 32), div_up(n, 32), batch), 256, 0, stream>>>(img, imgT, n);
        fp_dd_f32<<<grid, kDdThreads, 0, stream>>>(img, imgT, proj, sc, bo, usex, p->ns, p->na, n, p->dx, p->dy,
                                                   is, ps);
        st = check_launch("fp_par_2d distance driven");
        cudaFreeAsync(imgT, stream);  // after the kernel that reads it
        return st;
    }
}

template <typename T>
int dd_grad(const ctr_par_param* p, const T* proj, T* img, const double* w, const double* pos, const int* usex,
            int batch, cudaStream_t stream)
{
    int st = check_dd(p, proj, img, w, pos, usex, batch);
    if (st) return st;
    const unsigned long long pix = static_cast<unsigned long long>(p->nx) * p->ny;
    if constexpr (sizeof(T) == 8) {
        fp_dd_grad_kernel<T><<<dim3(div_up(pix, kDdThreads), batch), kDdThreads, 0, stream>>>(
            proj, img, w, pos, usex, p->ns, p->na, p->nx, p->ny, static_cast<size_t>(p->nx) * p->ny,
            static_cast<size_t>(p->na) * p->ns);
        return check_launch("fp_par_2d distance-driven grad");
    } else {
        // the fixed-point table and FP32 weights of this call (stream-ordered scratch)
        const size_t n_fx = static_cast<size_t>(p->na) * p->nx;
        char* scratch = nullptr;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&scratch),
                                        sizeof(DdGradFx) * n_fx + sizeof(float) * p->na, stream);
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "distance-driven grad scratch: %s", cudaGetErrorString(e));
        DdGradFx* fx = reinterpret_cast<DdGradFx*>(scratch);
        float* wf = reinterpret_cast<float*>(fx + n_fx);
        dd_grad_fx_prep<<<div_up(n_fx > p->na ? n_fx : p->na, 256), 256, 0, stream>>>(pos, w, fx, wf, p->na, p->nx);
        fp_dd_grad_f32<<<dim3(div_up(pix, kDdThreads), batch), kDdThreads, 0, stream>>>(
            proj, img, pos, fx, wf, usex, p->ns, p->na, p->nx, p->ny, static_cast<size_t>(p->nx) * p->ny,
            static_cast<size_t>(p->na) * p->ns);
        st = check_launch("fp_par_2d distance-driven grad");
        cudaFreeAsync(scratch, stream);  // after the kernels that read it
        return st;
    }
}

bool dd_views_along_x(double angle)
{
    return !((angle >= kDdPi / 4 && angle < 3 * kDdPi / 4) || (angle >= 5 * kDdPi / 4 && angle < 7 * kDdPi / 4));
}

template <typename V>
int dd_upload(V* dst, const std::vector<V>& src, cudaStream_t stream)
{
    cudaError_t e = cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(V), cudaMemcpyHostToDevice, stream);
    // the host vector dies on return: wait for the staged copy to leave it
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e == cudaSuccess ? CTR_OK : fail(CTR_ERR_CUDA, "distance-driven tables: %s", cudaGetErrorString(e));
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_fp_par_2d_dd_prep(const ctr_par_param* p, double* sincostbl, double* beginoffset, int* usex,
                          cudaStream_t stream)
{
    // reference src/fp_par_2d.cc:396-452 (running angle wrapped into [0, 2pi))
    if (!p || bad_ptr(sincostbl) || bad_ptr(beginoffset) || bad_ptr(usex))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->ns < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    const double centx = static_cast<double>(p->nx - 1) / 2.0 + p->offset_x;
    const double centy = static_cast<double>(p->ny - 1) / 2.0 + p->offset_y;
    const double cents = static_cast<double>(p->ns - 1) / 2.0 + p->offset_s;
    std::vector<double> sc(2 * static_cast<size_t>(p->na)), bo(static_cast<size_t>(p->na) * p->ns * 3);
    std::vector<int> ux(p->na);
    double angle = p->orbit_start;
    for (unsigned ia = 0; ia < p->na; ++ia) {
        while (angle < 0) angle += 2 * kDdPi;
        while (angle >= 2 * kDdPi) angle -= 2 * kDdPi;
        const double sa = std::sin(angle), ca = std::cos(angle);
        sc[2 * ia] = sa;
        sc[2 * ia + 1] = ca;
        ux[ia] = dd_views_along_x(angle) ? 1 : 0;
        double step, chan, begin;
        if (ux[ia]) {
            step = p->dy * sa / (ca * p->dx);
            chan = p->ds / (ca * p->dx);
            begin = centx - centy * step - cents * chan;
        } else {
            step = p->dx * ca / (sa * p->dy);
            chan = -p->ds / (sa * p->dy);
            begin = centy - centx * step - cents * chan;
        }
        for (unsigned is = 0; is < p->ns; ++is) {
            const size_t r = (static_cast<size_t>(ia) * p->ns + is) * 3;
            bo[r] = begin;
            bo[r + 1] = step;
            bo[r + 2] = chan / 2;
            begin += chan;
        }
        angle += p->orbit;
    }
    int st = dd_upload(sincostbl, sc, stream);
    if (st == CTR_OK) st = dd_upload(beginoffset, bo, stream);
    if (st == CTR_OK) st = dd_upload(usex, ux, stream);
    return st;
}

int ctr_fp_par_2d_dd_grad_prep(const ctr_par_param* p, double* weights, double* pos, int* usex,
                               cudaStream_t stream)
{
    // reference src/fp_par_2d.cc:547-596 (the angle is not wrapped here)
    if (!p || bad_ptr(weights) || bad_ptr(pos) || bad_ptr(usex)) return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->ns < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (p->nx != p->ny) return fail(CTR_ERR_INVALID_ARG, "distance-driven projection needs nx == ny");
    const double centx = static_cast<double>(p->nx - 1) / 2.0 + p->offset_x;
    const double centy = static_cast<double>(p->ny - 1) / 2.0 + p->offset_y;
    const double cents = static_cast<double>(p->ns - 1) / 2.0 + p->offset_s;
    std::vector<double> w(p->na), ps(static_cast<size_t>(p->na) * p->nx * 2);
    std::vector<int> ux(p->na);
    double angle = p->orbit_start;
    for (unsigned ia = 0; ia < p->na; ++ia) {
        const double sa = std::sin(angle), ca = std::cos(angle);
        ux[ia] = dd_views_along_x(angle) ? 1 : 0;
        double begin, o1, o2;
        if (ux[ia]) {
            w[ia] = std::fabs(p->dy / ca);
            o1 = p->dx * ca / p->ds;
            o2 = -p->dy * sa / p->ds;
            begin = cents - centx * o1 - centy * o2;
        } else {
            w[ia] = std::fabs(p->dx / sa);
            o1 = -p->dy * sa / p->ds;
            o2 = p->dx * ca / p->ds;
            begin = cents - centy * o1 - centx * o2;
        }
        for (unsigned i = 0; i < p->nx; ++i) {
            const size_t r = (static_cast<size_t>(ia) * p->nx + i) * 2;
            ps[r] = begin;
            ps[r + 1] = o1;
            begin += o2;
        }
        angle += p->orbit;
    }
    int st = dd_upload(weights, w, stream);
    if (st == CTR_OK) st = dd_upload(pos, ps, stream);
    if (st == CTR_OK) st = dd_upload(usex, ux, stream);
    return st;
}

int ctr_fp_par_2d_dd_f32(const ctr_par_param* p, const float* img, float* proj, const double* sincostbl,
                         const double* beginoffset, const int* usex, int batch, cudaStream_t stream)
{
    return dd_forward<float>(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}
int ctr_fp_par_2d_dd_f64(const ctr_par_param* p, const double* img, double* proj, const double* sincostbl,
                         const double* beginoffset, const int* usex, int batch, cudaStream_t stream)
{
    return dd_forward<double>(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}
int ctr_fp_par_2d_dd_grad_f32(const ctr_par_param* p, const float* proj, float* img, const double* weights,
                              const double* pos, const int* usex, int batch, cudaStream_t stream)
{
    return dd_grad<float>(p, proj, img, weights, pos, usex, batch, stream);
}
int ctr_fp_par_2d_dd_grad_f64(const ctr_par_param* p, const double* proj, double* img, const double* weights,
                              const double* pos, const int* usex, int batch, cudaStream_t stream)
{
    return dd_grad<double>(p, proj, img, weights, pos, usex, batch, stream);
}

}  // extern "C"
