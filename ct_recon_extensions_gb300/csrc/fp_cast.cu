// Ray-casting parallel forward projection: the reference's
// ParallelProjection2DRayCasting (src/fp_par_2d.cc:18-145).
//
// A ray enters the FoV circle (radius fov) at (x1, y1) in pixel-index units
// and takes nsteps samples of step step_size pixels along (sin t, cos t); a
// sample at the FP64 running position (x1 + sx + sx + ..., y1 + sy + ...) is
// used iff 0 <= x <= nx-1 and 0 <= y <= ny-1, and adds the bilinear
// interpolation of its four neighbours (floor / ceil corners).  The ray sum is
// scaled by step_size * dx.
//
// FP32 path (see fp_cast_f32 for the warp layout).  The sample range of each axis is decided
// exactly as the reference decides it: in 32.32 fixed point where that is
// certain, and by the reference's own FP64 accumulation (acc_advance, jumping
// binade to binade) for the few samples within a hair of an image edge
// (fp_setup.cuh).  The running position is monotone in k, so each axis keeps a
// contiguous range and the ray keeps their intersection.  Inside it the thread
// marches both coordinates in fixed point (two 64-bit adds a sample) and
// interpolates in FP32; positions differ from the reference's FP64 ones by
// ~1e-9 pixel, which moves the interpolation weights by as much (continuous at
// pixel boundaries).
//
// FP64 path: one thread per ray, the reference's loop (FP64 positions and
// inclusion test, FP64 interpolation and sum).
#include <cmath>
#include <vector>

#include "ctr_common.cuh"
#include "fp_setup.cuh"

namespace ctr {
namespace {

constexpr int kCastThreads = 128;

// Fraction of a 32.32 fixed-point value, from its low word's top 23 bits.
__device__ __forceinline__ float cast_frac(long long X)
{
    return __uint_as_float(0x3F800000u | (static_cast<unsigned>(X) >> 9)) - 1.0f;
}

// The FP32 kernel: a warp takes 32 consecutive rays.  Each lane first sets up
// one of them (sample range and fixed-point lines), then the warp marches the
// rays one after the other, lane l taking samples k0 + l, k0 + l + 32, ...: a
// warp's 32 samples lie within ~4 pixels of each other, so the four corner
// loads of a step touch a couple of cache lines instead of 32.  Each lane sums
// its samples in FP32, and a fixed shuffle tree adds the 32 lane sums.
__global__ void __launch_bounds__(kCastThreads)
    fp_cast_f32(const float* __restrict__ img, float* __restrict__ proj, const double* __restrict__ sincos,
                const double* __restrict__ begins, const int* __restrict__ nsteps, int ns, int na, int nx,
                int ny, double step_size, float scale, size_t img_stride, size_t proj_stride)
{
    const long long rays = static_cast<long long>(na) * ns;
    const int lane = threadIdx.x & 31;
    const long long r0 = (static_cast<long long>(blockIdx.x) * kCastThreads + threadIdx.x) - lane;
    if (r0 >= rays) return;  // warp-uniform
    // ---- set-up: lane l, ray r0 + l
    const long long ray = r0 + lane;
    long long X0 = 0, SX = 0, Y0 = 0, SY = 0;
    int k0 = 0, k1 = -1;
    if (ray < rays) {
        const int nstep = nsteps[ray];
        if (nstep > 0) {
            const int ia = static_cast<int>(ray / ns);
            const double sx = step_size * sincos[2 * ia], sy = step_size * sincos[2 * ia + 1];
            int kx0, kx1, ky0, ky1;
            axis_range(begins[2 * ray], sx, nstep, nx, &X0, &SX, &kx0, &kx1);
            axis_range(begins[2 * ray + 1], sy, nstep, ny, &Y0, &SY, &ky0, &ky1);
            k0 = max(kx0, ky0);
            k1 = min(kx1, ky1);
        }
    }
    const float* I = img + blockIdx.y * img_stride;
    float* out = proj + blockIdx.y * proj_stride;
    const int nr = static_cast<int>(min(32ll, rays - r0));
    for (int j = 0; j < nr; ++j) {
        const int a = __shfl_sync(0xffffffffu, k0, j), b = __shfl_sync(0xffffffffu, k1, j);
        const long long xs = __shfl_sync(0xffffffffu, SX, j), ys = __shfl_sync(0xffffffffu, SY, j);
        long long x = __shfl_sync(0xffffffffu, X0, j) + static_cast<long long>(a + lane) * xs;
        long long y = __shfl_sync(0xffffffffu, Y0, j) + static_cast<long long>(a + lane) * ys;
        const long long xs32 = xs * 32, ys32 = ys * 32;
        float part = 0.0f;
        for (int k = a + lane; k <= b; k += 32) {
            // exact positions are inside; the fixed-point ones may sit a hair
            // outside an edge: clamp the corner (the weight there is ~0)
            const int xi = static_cast<int>(x >> 32), yi = static_cast<int>(y >> 32);
            const int ix = min(max(xi, 0), nx - 1), iy = min(max(yi, 0), ny - 1);
            const float u = xi == ix ? cast_frac(x) : 0.0f, v = yi == iy ? cast_frac(y) : 0.0f;
            const int ix2 = min(ix + 1, nx - 1);
            const float* q1 = I + static_cast<size_t>(iy) * nx;
            const float* q2 = I + static_cast<size_t>(min(iy + 1, ny - 1)) * nx;
            const float a0 = __ldg(q1 + ix), a1 = __ldg(q1 + ix2);
            const float b0 = __ldg(q2 + ix), b1 = __ldg(q2 + ix2);
            const float p = fmaf(u, a1 - a0, a0), q = fmaf(u, b1 - b0, b0);
            part += fmaf(v, q - p, p);
            x += xs32;
            y += ys32;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == j) out[r0 + j] = part * scale;
    }
}

__global__ void __launch_bounds__(kCastThreads)
    fp_cast_f64(const double* __restrict__ img, double* __restrict__ proj, const double* __restrict__ sincos,
                const double* __restrict__ begins, const int* __restrict__ nsteps, int ns, int na, int nx,
                int ny, double step_size, double dx, size_t img_stride, size_t proj_stride)
{
    const long long ray = static_cast<long long>(blockIdx.x) * kCastThreads + threadIdx.x;
    if (ray >= static_cast<long long>(na) * ns) return;
    const int ia = static_cast<int>(ray / ns);
    double* out = proj + blockIdx.y * proj_stride + ray;
    const int nstep = nsteps[ray];
    if (nstep <= 0) {
        *out = 0.0;
        return;
    }
    const double sx = step_size * sincos[2 * ia], sy = step_size * sincos[2 * ia + 1];
    const double xmax = static_cast<double>(nx - 1), ymax = static_cast<double>(ny - 1);
    const double* I = img + blockIdx.y * img_stride;
    double x = begins[2 * ray], y = begins[2 * ray + 1], sum = 0.0;
    for (int k = 0; k < nstep; ++k) {
        if (x >= 0 && x <= xmax && y >= 0 && y <= ymax) {
            const int ix1 = static_cast<int>(floor(x)), ix2 = static_cast<int>(ceil(x));
            const int iy1 = static_cast<int>(floor(y)), iy2 = static_cast<int>(ceil(y));
            const double u = x - ix1, v = y - iy1;
            const double* r1 = I + static_cast<size_t>(iy1) * nx;
            const double* r2 = I + static_cast<size_t>(iy2) * nx;
            sum += (1 - v) * ((1 - u) * r1[ix1] + u * r1[ix2]) + v * ((1 - u) * r2[ix1] + u * r2[ix2]);
        }
        x += sx;
        y += sy;
    }
    *out = sum * step_size * dx;
}

int check_cast(const ctr_par_param* p, double step_size, const void* a, const void* b, const void* sc,
               const void* begins, const void* nsteps, int batch)
{
    if (!p || bad_ptr(a) || bad_ptr(b) || bad_ptr(sc) || bad_ptr(begins) || bad_ptr(nsteps))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (p->ns < 1 || p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (!(step_size > 0.0)) return fail(CTR_ERR_INVALID_ARG, "step_size must be positive");
    if (batch > 65535) return fail(CTR_ERR_UNSUPPORTED, "batch > 65535");
    if (a == b) return fail(CTR_ERR_INVALID_ARG, "projection cannot run in place");
    return CTR_OK;
}

template <typename T>
int cast_forward(const ctr_par_param* p, double step_size, const T* img, T* proj, const double* sc,
                 const double* begins, const int* nsteps, int batch, cudaStream_t stream)
{
    int st = check_cast(p, step_size, img, proj, sc, begins, nsteps, batch);
    if (st) return st;
    const long long rays = static_cast<long long>(p->na) * p->ns;
    const dim3 grid(static_cast<unsigned>(div_up(static_cast<unsigned long long>(rays), kCastThreads)), batch);
    const size_t is = static_cast<size_t>(p->nx) * p->ny, ps = static_cast<size_t>(p->na) * p->ns;
    if constexpr (sizeof(T) == 4)
        fp_cast_f32<<<grid, kCastThreads, 0, stream>>>(img, proj, sc, begins, nsteps, p->ns, p->na, p->nx, p->ny,
                                                       step_size, static_cast<float>(step_size * p->dx), is, ps);
    else
        fp_cast_f64<<<grid, kCastThreads, 0, stream>>>(img, proj, sc, begins, nsteps, p->ns, p->na, p->nx, p->ny,
                                                       step_size, p->dx, is, ps);
    return check_launch("fp_par_2d ray casting");
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_fp_par_2d_cast_prep(const ctr_par_param* p, double step_size, double* sincostbl, double* begins,
                            int* nsteps, cudaStream_t stream)
{
    // reference src/fp_par_2d.cc:18-80: running angle and channel coordinate
    // (angle += orbit, s += ds), the angle not wrapped
    if (!p || bad_ptr(sincostbl) || bad_ptr(begins) || bad_ptr(nsteps))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->ns < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (!(step_size > 0.0)) return fail(CTR_ERR_INVALID_ARG, "step_size must be positive");
    const double xc = static_cast<double>(p->nx - 1) / 2.0 + p->offset_x;
    const double yc = static_cast<double>(p->ny - 1) / 2.0 + p->offset_y;
    const double fov2 = p->fov * p->fov;
    const double s0 = -(static_cast<double>(p->ns - 1) / 2.0 + p->offset_s) * p->ds;
    const size_t rays = static_cast<size_t>(p->na) * p->ns;
    std::vector<double> sc(2 * static_cast<size_t>(p->na)), bg(2 * rays);
    std::vector<int> nst(rays);
    double angle = p->orbit_start;
    for (unsigned ia = 0; ia < p->na; ++ia) {
        const double sa = std::sin(angle), ca = std::cos(angle);
        sc[2 * ia] = sa;
        sc[2 * ia + 1] = ca;
        const double sx = step_size * sa, sy = step_size * ca;
        const bool along_x = sa > (1.0 / 1.414);
        double s = s0;
        for (unsigned is = 0; is < p->ns; ++is) {
            const size_t r = static_cast<size_t>(ia) * p->ns + is;
            const double h2 = fov2 - s * s;
            if (h2 > 0) {
                const double h = std::sqrt(h2);
                const double x1 = (s * ca - h * sa) / p->dx + xc;
                const double y1 = -(s * sa + h * ca) / p->dy + yc;
                const double x2 = (s * ca + h * sa) / p->dx + xc;
                const double y2 = -(s * sa - h * ca) / p->dy + yc;
                nst[r] = along_x ? static_cast<int>((x2 - x1) / sx) : static_cast<int>((y2 - y1) / sy);
                bg[2 * r] = x1;
                bg[2 * r + 1] = y1;
            } else {
                nst[r] = 0;
                bg[2 * r] = 0;
                bg[2 * r + 1] = 0;
            }
            s += p->ds;
        }
        angle += p->orbit;
    }
    cudaError_t e = cudaMemcpyAsync(sincostbl, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(begins, bg.data(), bg.size() * sizeof(double), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(nsteps, nst.data(), nst.size() * sizeof(int), cudaMemcpyHostToDevice, stream);
    // the host vectors die on return: wait for the staged copies to leave them
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "ray-casting tables: %s", cudaGetErrorString(e));
    return CTR_OK;
}

int ctr_fp_par_2d_cast_f32(const ctr_par_param* p, double step_size, const float* img, float* proj,
                           const double* sincostbl, const double* begins, const int* nsteps, int batch,
                           cudaStream_t stream)
{
    return cast_forward<float>(p, step_size, img, proj, sincostbl, begins, nsteps, batch, stream);
}

int ctr_fp_par_2d_cast_f64(const ctr_par_param* p, double step_size, const double* img, double* proj,
                           const double* sincostbl, const double* begins, const int* nsteps, int batch,
                           cudaStream_t stream)
{
    return cast_forward<double>(p, step_size, img, proj, sincostbl, begins, nsteps, batch, stream);
}

}  // extern "C"
