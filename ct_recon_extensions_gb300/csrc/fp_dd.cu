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

namespace ctr {
namespace {

constexpr int kDdThreads = 128;
constexpr double kDdPi = 3.14159265358979323846;

template <typename T>
__global__ void __launch_bounds__(kDdThreads)
    fp_dd_kernel(const T* __restrict__ img, T* __restrict__ proj, const double* __restrict__ sincos,
                 const double* __restrict__ bo, const int* __restrict__ usex, int ns, int na, int nx, int ny,
                 double dx, double dy, size_t img_stride, size_t proj_stride)
{
    const long long ray = static_cast<long long>(blockIdx.x) * kDdThreads + threadIdx.x;
    if (ray >= static_cast<long long>(na) * ns) return;
    const int ia = static_cast<int>(ray / ns);
    const T* I = img + blockIdx.y * img_stride;
    const int ux = usex[ia];
    const double w = ux ? fabs(dy / sincos[2 * ia + 1]) : fabs(dx / sincos[2 * ia]);
    const int nl = ux ? ny : nx;    // lines
    const int nal = ux ? nx : ny;   // pixels along a line
    const size_t step_line = ux ? static_cast<size_t>(nx) : 1;   // next line
    const size_t step_pix = ux ? 1 : static_cast<size_t>(nx);    // next pixel along the line
    const double* b = bo + 3 * ray;
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
            // intervals i0 .. i1 (i < cr), all but those from nal - 1 on
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
    proj[blockIdx.y * proj_stride + ray] = static_cast<T>(sum * w);
}

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
    using Acc = typename std::conditional<sizeof(T) == 4, float, double>::type;
    Acc sum = 0;
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
        Acc tmp = 0;
        for (int is = static_cast<int>(fmin(c0, last + 1.0)); static_cast<double>(is) <= last; ++is) {
            const double hi = __dadd_rn(static_cast<double>(is), 0.5), lo = __dsub_rn(static_cast<double>(is), 0.5);
            const double len = __dsub_rn(hi < right ? hi : right, lo > left ? lo : left);
            const size_t k = static_cast<size_t>(ia) * ns + is;
            const T p = k < total ? P[k] : static_cast<T>(0);
            if constexpr (sizeof(T) == 4) tmp = fmaf(static_cast<float>(len), p * 0.5f, tmp);
            else tmp += len * p / 2;
        }
        if constexpr (sizeof(T) == 4) sum = fmaf(tmp, static_cast<float>(weights[ia]), sum);
        else sum += tmp * weights[ia];
    }
    img[blockIdx.y * img_stride + pix] = static_cast<T>(sum);
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
    fp_dd_kernel<T><<<dim3(div_up(rays, kDdThreads), batch), kDdThreads, 0, stream>>>(
        img, proj, sc, bo, usex, p->ns, p->na, p->nx, p->ny, p->dx, p->dy,
        static_cast<size_t>(p->nx) * p->ny, static_cast<size_t>(p->na) * p->ns);
    return check_launch("fp_par_2d distance driven");
}

template <typename T>
int dd_grad(const ctr_par_param* p, const T* proj, T* img, const double* w, const double* pos, const int* usex,
            int batch, cudaStream_t stream)
{
    int st = check_dd(p, proj, img, w, pos, usex, batch);
    if (st) return st;
    const unsigned long long pix = static_cast<unsigned long long>(p->nx) * p->ny;
    fp_dd_grad_kernel<T><<<dim3(div_up(pix, kDdThreads), batch), kDdThreads, 0, stream>>>(
        proj, img, w, pos, usex, p->ns, p->na, p->nx, p->ny, static_cast<size_t>(p->nx) * p->ny,
        static_cast<size_t>(p->na) * p->ns);
    return check_launch("fp_par_2d distance-driven grad");
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
