// The reference's numpy extension ABI (numpy_ext/common.cu:29-61,
// numpy_ext/fan_weighting_npext.cu:86-106, numpy_ext/filter_npext.cu:104-124,
// numpy_ext/bp_fan_2d_angle_npext.cu:136-159): the same extern "C" names and
// signatures, handle-based, on HOST double arrays.  Each run copies the input
// to the device, runs the FP64 kernels of this library on the selected
// device's stream, copies the result back and synchronises, as the reference
// does.  Differences by design: no C++ exception crosses the ABI (failures
// return false / -1, with ctr_last_error()); set_device(-1) (the reference's
// CPU mode) is refused because this library is the GPU implementation only;
// angles are copied at create time (the reference keeps the caller's pointer).
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "ctr_common.cuh"

namespace ctr {
namespace {

std::mutex g_mu;
int g_device = -1;
cudaStream_t g_stream = nullptr;

struct DevBuf {
    double* p = nullptr;
    size_t n = 0;
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    bool ensure(size_t count)
    {
        if (p && n >= count) return true;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, count * sizeof(double)) != cudaSuccess) return false;
        n = count;
        return true;
    }
};

struct FanWeightingHandle {
    ctr_fan_weighting_param p;
    DevBuf buf;
};

struct RampFilterHandle {
    ctr_filter_param p;
    DevBuf in, out, taps;
    bool prepared = false;
};

struct FanBpAngleHandle {
    ctr_fan_bp_angle_param p;
    std::vector<double> angles;
    DevBuf in, out, xpos, ypos, sc, dang;
    bool prepared = false;
};

template <class H>
struct Registry {
    std::map<int, std::unique_ptr<H>> items;
    int count = 0;
    int add(std::unique_ptr<H> h)
    {
        items.emplace(++count, std::move(h));
        return count;
    }
    H* get(int id)
    {
        auto it = items.find(id);
        return it == items.end() ? nullptr : it->second.get();
    }
    bool erase(int id) { return items.erase(id) > 0; }
};

Registry<FanWeightingHandle> g_fw;
Registry<RampFilterHandle> g_rf;
Registry<FanBpAngleHandle> g_bp;

bool ready()
{
    if (g_device < 0 || !g_stream) {
        fail(CTR_ERR_DEVICE, "call set_device(device >= 0) first");
        return false;
    }
    return cudaSetDevice(g_device) == cudaSuccess;
}

bool h2d(double* dst, const double* src, size_t n)
{
    return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, g_stream) ==
           cudaSuccess;
}

bool d2h_sync(double* dst, const double* src, size_t n)
{
    if (cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, g_stream) !=
        cudaSuccess)
        return false;
    const cudaError_t e = cudaStreamSynchronize(g_stream);
    if (e != cudaSuccess) fail(CTR_ERR_CUDA, "%s", cudaGetErrorString(e));
    return e == cudaSuccess;
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

bool set_device(const int device)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (device < 0) {
        fail(CTR_ERR_UNSUPPORTED, "set_device(%d): this library has no CPU mode", device);
        return false;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        fail(CTR_ERR_DEVICE, "Device not found!");
        return false;
    }
    if (ctr_device_check() != CTR_OK) return false;
    if (g_stream && g_device != device) {
        cudaStreamDestroy(g_stream);
        g_stream = nullptr;
    }
    if (!g_stream && cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking) != cudaSuccess) {
        fail(CTR_ERR_CUDA, "Stream initialization failed!");
        return false;
    }
    g_device = device;
    return true;
}

bool clear()
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_stream) cudaStreamDestroy(g_stream);
    g_stream = nullptr;
    return true;
}

// ---- fan weighting --------------------------------------------------------
int fan_weighting_create(unsigned int ns, unsigned int nrow, double ds, double offset, double dso,
                         double dsd, int type)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto h = std::make_unique<FanWeightingHandle>();
    h->p = ctr_fan_weighting_param{ns, nrow, ds, offset, dso, dsd, type};
    return g_fw.add(std::move(h));
}

bool fan_weighting_run(int handle, double* in, double* out)
{
    std::lock_guard<std::mutex> lock(g_mu);
    FanWeightingHandle* h = g_fw.get(handle);
    if (!h || !in || !out || !ready()) return false;
    const size_t n = static_cast<size_t>(h->p.ns) * h->p.nrow;
    if (!h->buf.ensure(n) || !h2d(h->buf.p, in, n)) return false;
    if (ctr_fan_weighting_f64(&h->p, h->buf.p, h->buf.p, 1, g_stream) != CTR_OK) return false;
    return d2h_sync(out, h->buf.p, n);
}

bool fan_weighting_destroy(int handle)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return g_fw.erase(handle);
}

// ---- ramp filter ----------------------------------------------------------
int ramp_filter_create(unsigned int ns, unsigned int nrow, double ds, double dsd, int type)
{
    std::lock_guard<std::mutex> lock(g_mu);
    auto h = std::make_unique<RampFilterHandle>();
    h->p = ctr_filter_param{ns, nrow, ds, dsd, type, 0};
    return g_rf.add(std::move(h));
}

bool ramp_filter_run(int handle, double* in, double* out)
{
    std::lock_guard<std::mutex> lock(g_mu);
    RampFilterHandle* h = g_rf.get(handle);
    if (!h || !in || !out || !ready()) return false;
    const size_t n = static_cast<size_t>(h->p.ns) * h->p.nrow;
    if (!h->prepared) {
        if (!h->taps.ensure(2 * h->p.ns + 1) ||
            ctr_ramp_filter_prep(&h->p, h->taps.p, g_stream) != CTR_OK)
            return false;
        h->prepared = true;
    }
    if (!h->in.ensure(n) || !h->out.ensure(n) || !h2d(h->in.p, in, n)) return false;
    if (ctr_ramp_filter_f64(&h->p, h->in.p, h->taps.p, h->out.p, 1, g_stream) != CTR_OK)
        return false;
    return d2h_sync(out, h->out.p, n);
}

bool ramp_filter_destroy(int handle)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return g_rf.erase(handle);
}

// ---- fan backprojection with an angle list ----------------------------------
int fan_bp_2d_angle_create(double* angles, unsigned int ns, unsigned int na, double ds,
                           double offset_s, unsigned int nx, unsigned int ny, double dx, double dy,
                           double offset_x, double offset_y, double dso, double dsd, double fov)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!angles) {
        fail(CTR_ERR_INVALID_ARG, "angles is null");
        return -1;
    }
    auto h = std::make_unique<FanBpAngleHandle>();
    h->p = ctr_fan_bp_angle_param{ns, na, ds, offset_s, nx, ny, dx, dy, offset_x, offset_y, dso,
                                  dsd, fov};
    h->angles.assign(angles, angles + na);
    return g_bp.add(std::move(h));
}

bool fan_bp_2d_angle_run(int handle, double* in, double* out)
{
    std::lock_guard<std::mutex> lock(g_mu);
    FanBpAngleHandle* h = g_bp.get(handle);
    if (!h || !in || !out || !ready()) return false;
    if (!h->prepared) {
        if (!h->xpos.ensure(h->p.nx) || !h->ypos.ensure(h->p.ny) || !h->sc.ensure(2 * h->p.na) ||
            !h->dang.ensure(h->p.na) || !h2d(h->dang.p, h->angles.data(), h->p.na))
            return false;
        if (ctr_bp_fan_2d_angle_prep(&h->p, h->dang.p, h->xpos.p, h->ypos.p, h->sc.p, g_stream) !=
            CTR_OK)
            return false;
        h->prepared = true;
    }
    const size_t ni = static_cast<size_t>(h->p.ns) * h->p.na;
    const size_t no = static_cast<size_t>(h->p.nx) * h->p.ny;
    if (!h->in.ensure(ni) || !h->out.ensure(no) || !h2d(h->in.p, in, ni)) return false;
    if (ctr_bp_fan_2d_angle_f64(&h->p, h->in.p, h->out.p, h->xpos.p, h->ypos.p, h->sc.p, 1,
                                g_stream) != CTR_OK)
        return false;
    return d2h_sync(out, h->out.p, no);
}

bool fan_bp_2d_angle_destroy(int handle)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return g_bp.erase(handle);
}

}  // extern "C"
