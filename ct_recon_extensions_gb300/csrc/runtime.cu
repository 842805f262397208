// Runtime pieces of the C ABI: status strings, per-thread error messages,
// device checks, kernel self-check flags and the geometry-table preps.
//
// The preps reproduce the reference's Prep::calculate_on_cpu arithmetic in
// FP64 on the host (angles by repeated addition, positions by repeated
// addition) and copy the tables to the caller's device buffers in stream
// order, so GPU tables are bit-identical to the reference's CPU tables.
#include <cstdarg>
#include <cstring>
#include <vector>

#include "ctr_async.cuh"
#include "ctr_common.cuh"
#include "host_geometry.h"

namespace ctr {

__device__ unsigned int g_kernel_flags = 0;

namespace {
thread_local char t_last_error[512] = {0};

constexpr double kPi = 3.14159265358979323846;
constexpr double kPi4 = 0.78539816339744830962;

template <typename V>
int upload(V* dst, const std::vector<V>& src, cudaStream_t stream, const char* what)
{
    cudaError_t e = cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(V),
                                    cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    // the host vector dies on return: wait for the staged copy to leave it
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return CTR_OK;
}

bool views_along_x(double angle)
{
    return !((angle >= kPi4 && angle < 3 * kPi4) || (angle >= 5 * kPi4 && angle < 7 * kPi4));
}
}  // namespace

void pixel_positions(unsigned nx, unsigned ny, double dx, double dy, double ox, double oy,
                     std::vector<double>& xpos, std::vector<double>& ypos)
{
    const double centx = static_cast<double>(nx - 1) / 2 + ox;
    const double centy = static_cast<double>(ny - 1) / 2 + oy;
    xpos.resize(nx);
    ypos.resize(ny);
    double posx = -centx * dx, posy = centy * dy;
    for (unsigned i = 0; i < nx; ++i) {
        xpos[i] = posx;
        posx += dx;
    }
    for (unsigned i = 0; i < ny; ++i) {
        ypos[i] = posy;
        posy -= dy;
    }
}

void fan_sincos(unsigned na, double orbit_start, double orbit, std::vector<double>& sc)
{
    sc.resize(2 * static_cast<size_t>(na));
    double angle = orbit_start;
    for (unsigned ia = 0; ia < na; ++ia) {
        sc[2 * ia] = std::sin(angle);
        sc[2 * ia + 1] = std::cos(angle);
        angle += orbit;
    }
}

bool ramp_taps(unsigned ns, double ds, double dsd, int type, std::vector<double>& taps)
{
    const int n = static_cast<int>(ns);
    taps.assign(2 * static_cast<size_t>(n) + 1, 0.0);
    double* h = taps.data() + n;
    if (type == 0 || type == 2) {
        const double ds2_inv = 1.0 / (ds * ds);
        const double pi2_inv = 1.0 / (kPi * kPi);
        for (int k = -n; k <= n; ++k)
            h[k] = k == 0 ? 0.25 * ds2_inv
                          : (k % 2 == 0 ? 0.0 : -pi2_inv * ds2_inv / static_cast<double>(k * k));
        return true;
    }
    if (type == 1) {
        const double pidsd2_inv = 1.0 / (kPi * kPi * dsd * dsd);
        for (int k = -n; k <= n; ++k) {
            if (k == 0) {
                h[k] = 0.25 / (ds * ds);
            } else if (k % 2 == 0) {
                h[k] = 0.0;
            } else {
                const double sa = std::sin(static_cast<double>(k) * ds / dsd);
                h[k] = -pidsd2_inv / (sa * sa);
            }
        }
        return true;
    }
    return false;
}

bool fan_weights(unsigned ns, double ds, double offset, double dso, double dsd, int type,
                 std::vector<double>& w)
{
    if (type != 1 && type != 2) return false;
    w.resize(ns);
    const double cents = static_cast<double>(ns - 1) / 2 + offset;
    for (unsigned is = 0; is < ns; ++is) {
        const double s = ds * (static_cast<double>(is) - cents);
        w[is] = type == 2 ? dso * std::fabs(std::cos(std::atan2(s, dsd))) / dsd
                          : dso * std::fabs(std::cos(s / dsd)) / dsd;
    }
    return true;
}

int fail(int status, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_last_error, sizeof(t_last_error), fmt, ap);
    va_end(ap);
    return status;
}

int check_launch(const char* what)
{
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return CTR_OK;
    if (e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDeviceFunction)
        return fail(CTR_ERR_DEVICE, "%s: %s (this library is built for sm_103a only)", what,
                    cudaGetErrorString(e));
    return fail(CTR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int check_common(int batch)
{
    if (batch < 1) return fail(CTR_ERR_INVALID_ARG, "batch must be >= 1 (got %d)", batch);
    return CTR_OK;
}

}  // namespace ctr

using namespace ctr;

extern "C" {

const char* ctr_status_string(int status)
{
    switch (status) {
    case CTR_OK: return "ok";
    case CTR_ERR_INVALID_ARG: return "invalid argument";
    case CTR_ERR_UNSUPPORTED: return "unsupported";
    case CTR_ERR_CUDA: return "CUDA runtime error";
    case CTR_ERR_DEVICE: return "no usable sm_103 device";
    case CTR_ERR_KERNEL: return "kernel self-check failed";
    default: return "unknown status";
    }
}

const char* ctr_last_error(void) { return t_last_error; }

int ctr_version(void) { return 10000; }

int ctr_device_check(void)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(CTR_ERR_DEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess)
        return fail(CTR_ERR_DEVICE, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
    if (prop.major != 10 || prop.minor != 3)
        return fail(CTR_ERR_DEVICE, "device %d is sm_%d%d; this library needs sm_103", dev,
                    prop.major, prop.minor);
    return CTR_OK;
}

// Self-test of the bounded-wait error path (see the header): one CTA arms an
// mbarrier for a 16-byte copy that is never issued, as a producer that
// skipped its stage would, and waits on it with the library's bounded wait
// under `limit_ns`; the wait runs out, the kernel raises kFlagWaitTimeout and
// returns.  No copy is in flight when it exits.
__global__ void selftest_wait_kernel(unsigned long long limit_ns, int* waited_out)
{
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_expect_tx(smem_u32(&bar), 16);  // the copy that never comes
    __syncthreads();
    const bool ok = mbar_wait_bounded(smem_u32(&bar), 0, limit_ns);
    if (!ok && threadIdx.x == 0) {
        raise_flag(kFlagWaitTimeout);
        *waited_out = 1;
    }
}

int ctr_selftest_wait_timeout(unsigned long long limit_ns, cudaStream_t stream)
{
    if (limit_ns == 0 || limit_ns > kWaitLimitNs) return fail(CTR_ERR_INVALID_ARG, "limit_ns must be in (0, 1 s]");
    int* waited = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&waited), sizeof(int), stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "self-test: %s", cudaGetErrorString(e));
    e = cudaMemsetAsync(waited, 0, sizeof(int), stream);
    if (e == cudaSuccess) {
        selftest_wait_kernel<<<1, 64, 0, stream>>>(limit_ns, waited);
        e = cudaGetLastError();
    }
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, waited, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    cudaFreeAsync(waited, stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "self-test: %s", cudaGetErrorString(e));
    unsigned int flags = 0;
    int st = ctr_kernel_flags(&flags, 0);
    if (st) return st;
    if (h && (flags & kFlagWaitTimeout))
        return fail(CTR_ERR_KERNEL, "a bounded wait gave up after %llu ns (kernel flags 0x%x)", limit_ns, flags);
    return CTR_OK;
}

int ctr_kernel_flags(unsigned int* flags, int reset)
{
    if (!flags) return fail(CTR_ERR_INVALID_ARG, "flags is null");
    cudaError_t e = cudaMemcpyFromSymbol(flags, g_kernel_flags, sizeof(unsigned int));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "read flags: %s", cudaGetErrorString(e));
    if (reset) {
        unsigned int zero = 0;
        e = cudaMemcpyToSymbol(g_kernel_flags, &zero, sizeof(unsigned int));
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "reset flags: %s", cudaGetErrorString(e));
    }
    return CTR_OK;
}

// ---- preps -------------------------------------------------------------------

int ctr_ramp_filter_prep(const ctr_filter_param* p, double* filter, cudaStream_t stream)
{
    // reference src/filter.cc:18-65
    if (!p || bad_ptr(filter)) return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->ns < 1) return fail(CTR_ERR_INVALID_ARG, "ns must be >= 1");
    std::vector<double> taps;
    if (!ramp_taps(p->ns, p->ds, p->dsd, p->type, taps))
        return fail(CTR_ERR_INVALID_ARG, "ramp filter type %d (0 par, 1 fan, 2 flat)", p->type);
    return upload(filter, taps, stream, "ramp filter taps");
}

int ctr_bp_fan_2d_prep(const ctr_fan_bp_param* p, double* xpos, double* ypos,
                       double* sincostbl, cudaStream_t stream)
{
    // reference src/bp_fan_2d.cc:18-44
    if (!p || bad_ptr(xpos) || bad_ptr(ypos) || bad_ptr(sincostbl))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    std::vector<double> sc, xp, yp;
    fan_sincos(p->na, p->orbit_start, p->orbit, sc);
    pixel_positions(p->nx, p->ny, p->dx, p->dy, p->offset_x, p->offset_y, xp, yp);
    int st = upload(sincostbl, sc, stream, "sincostbl");
    if (st == CTR_OK) st = upload(xpos, xp, stream, "xpos");
    if (st == CTR_OK) st = upload(ypos, yp, stream, "ypos");
    return st;
}

int ctr_bp_fan_2d_angle_prep(const ctr_fan_bp_angle_param* p, const double* angles,
                             double* xpos, double* ypos, double* sincostbl,
                             cudaStream_t stream)
{
    // reference src/bp_fan_2d_angle.cc:18-45; angles is a device array
    if (!p || bad_ptr(angles) || bad_ptr(xpos) || bad_ptr(ypos) || bad_ptr(sincostbl))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    std::vector<double> ang(p->na), sc(2 * p->na), xp, yp;
    cudaError_t e = cudaMemcpyAsync(ang.data(), angles, p->na * sizeof(double),
                                    cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "read angles: %s", cudaGetErrorString(e));
    for (unsigned ia = 0; ia < p->na; ++ia) {
        sc[2 * ia] = std::sin(ang[ia]);
        sc[2 * ia + 1] = std::cos(ang[ia]);
    }
    pixel_positions(p->nx, p->ny, p->dx, p->dy, p->offset_x, p->offset_y, xp, yp);
    int st = upload(sincostbl, sc, stream, "sincostbl");
    if (st == CTR_OK) st = upload(xpos, xp, stream, "xpos");
    if (st == CTR_OK) st = upload(ypos, yp, stream, "ypos");
    return st;
}

int ctr_bp_par_2d_prep(const ctr_par_param* p, double* xcos, double* ysin, int* buffer,
                       cudaStream_t stream)
{
    // reference src/bp_par_2d.cc:18-49 (buffer unused)
    (void)buffer;
    if (!p || bad_ptr(xcos) || bad_ptr(ysin)) return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    const double centx = static_cast<double>(p->nx - 1) / 2 + p->offset_x;
    const double centy = static_cast<double>(p->ny - 1) / 2 + p->offset_y;
    std::vector<double> xc(static_cast<size_t>(p->nx) * p->na),
        ys(static_cast<size_t>(p->ny) * p->na);
    double angle = p->orbit_start;
    for (unsigned ia = 0; ia < p->na; ++ia) {
        const double sa = std::sin(angle), ca = std::cos(angle);
        double posx = -centx * p->dx;
        for (unsigned ix = 0; ix < p->nx; ++ix) {
            xc[ia + static_cast<size_t>(ix) * p->na] = posx * ca;
            posx += p->dx;
        }
        double posy = centy * p->dy;
        for (unsigned iy = 0; iy < p->ny; ++iy) {
            ys[ia + static_cast<size_t>(iy) * p->na] = posy * sa;
            posy -= p->dy;
        }
        angle += p->orbit;
    }
    int st = upload(xcos, xc, stream, "xcos");
    if (st == CTR_OK) st = upload(ysin, ys, stream, "ysin");
    return st;
}

int ctr_fp_par_2d_prep(const ctr_par_param* p, double* sincostbl, double* beginoffset,
                       int* usex, cudaStream_t stream)
{
    // reference src/fp_par_2d.cc:149-208 (running angle wrapped into [0, 2pi))
    if (!p || bad_ptr(sincostbl) || bad_ptr(beginoffset) || bad_ptr(usex))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->ns < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    const double centx = static_cast<double>(p->nx - 1) / 2.0 + p->offset_x;
    const double centy = static_cast<double>(p->ny - 1) / 2.0 + p->offset_y;
    const double cents = static_cast<double>(p->ns - 1) / 2.0 + p->offset_s;
    std::vector<double> sc(2 * p->na), bo(static_cast<size_t>(p->na) * p->ns * 2);
    std::vector<int> ux(p->na);
    double angle = p->orbit_start;
    for (unsigned ia = 0; ia < p->na; ++ia) {
        while (angle < 0) angle += 2 * kPi;
        while (angle >= 2 * kPi) angle -= 2 * kPi;
        const double sa = std::sin(angle), ca = std::cos(angle);
        sc[2 * ia] = sa;
        sc[2 * ia + 1] = ca;
        ux[ia] = views_along_x(angle) ? 1 : 0;
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
        double* b = bo.data() + static_cast<size_t>(ia) * p->ns * 2;
        for (unsigned is = 0; is < p->ns; ++is) {
            b[2 * is] = begin;
            b[2 * is + 1] = step;
            begin += chan;
        }
        angle += p->orbit;
    }
    int st = upload(sincostbl, sc, stream, "sincostbl");
    if (st == CTR_OK) st = upload(beginoffset, bo, stream, "beginoffset");
    if (st == CTR_OK) st = upload(usex, ux, stream, "usex");
    return st;
}

int ctr_fp_par_2d_grad_prep(const ctr_par_param* p, double* weights, double* pos, int* usex,
                            cudaStream_t stream)
{
    // reference src/fp_par_2d.cc:285-321 (the angle is not wrapped here)
    if (!p || bad_ptr(weights) || bad_ptr(pos) || bad_ptr(usex))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    if (p->na < 1 || p->nx < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (p->nx != p->ny) return fail(CTR_ERR_INVALID_ARG, "ray-driven projection needs nx == ny");
    const double centx = static_cast<double>(p->nx - 1) / 2.0 + p->offset_x;
    const double centy = static_cast<double>(p->ny - 1) / 2.0 + p->offset_y;
    const double cents = static_cast<double>(p->ns - 1) / 2.0 + p->offset_s;
    std::vector<double> w(p->na), ps(static_cast<size_t>(p->na) * p->nx * 2);
    std::vector<int> ux(p->na);
    double angle = p->orbit_start;
    double* pp = ps.data();
    for (unsigned ia = 0; ia < p->na; ++ia) {
        const double sa = std::sin(angle), ca = std::cos(angle);
        ux[ia] = views_along_x(angle) ? 1 : 0;
        if (ux[ia]) {
            w[ia] = std::fabs(p->dy / ca);
            const double o1 = p->dx * ca / p->ds, o2 = -p->dy * sa / p->ds;
            double begin = cents - centx * o1 - centy * o2;
            for (unsigned iy = 0; iy < p->ny; ++iy, pp += 2) {
                pp[0] = begin;
                pp[1] = o1;
                begin += o2;
            }
        } else {
            w[ia] = std::fabs(p->dx / sa);
            const double o1 = -p->dy * sa / p->ds, o2 = p->dx * ca / p->ds;
            double begin = cents - centy * o1 - centx * o2;
            for (unsigned ix = 0; ix < p->nx; ++ix, pp += 2) {
                pp[0] = begin;
                pp[1] = o1;
                begin += o2;
            }
        }
        angle += p->orbit;
    }
    int st = upload(weights, w, stream, "weights");
    if (st == CTR_OK) st = upload(pos, ps, stream, "pos");
    if (st == CTR_OK) st = upload(usex, ux, stream, "usex");
    return st;
}

}  // extern "C"
