// C++ mirror of the reference's include/helical_interpolation.h (lines 17-116):
// HelicalInterpolationParam, HelicalInterpolation360<T>, HelicalInterpolation180<T>.
//
// The reference implements these on the CPU only (calculate_on_cpu); here
// calculate_on_gpu runs the same rebinning on device buffers, input
// [na][nt][ns] and output [nz][view_per_rot][ns].  Like the reference it
// throws std::runtime_error("View not enough for this slice!") and
// std::runtime_error("No row data available!"); other failures return false.
// The call allocates its table and per-slice status words on `stream`,
// prepares the table on the host, runs and synchronises the stream.
#ifndef CT_RECON_GB300_HELICAL_INTERPOLATION_H_
#define CT_RECON_GB300_HELICAL_INTERPOLATION_H_

#include <stdexcept>
#include <string>
#include <vector>

#include "ct_recon/common.h"

namespace ct_recon {

struct HelicalInterpolationParam {
    unsigned int ns;       // channels
    unsigned int nt;       // detector rows
    unsigned int na;       // views
    double ds;             // channel spacing, mm
    double dt;             // row spacing, mm (unused, as in the reference)
    double offset_s;       // centre channel minus (ns-1)/2
    double offset_t;       // centre row minus (nt-1)/2
    double orbit_start;    // source angle of view 0 (unused, as in the reference)
    double orbit;          // angle between views
    double couch_begin;    // source z of view 0
    double couch_mov;      // source z step between views
    unsigned int view_per_rot;
    unsigned int nz;       // output slices
    double dz;             // slice spacing
    double z0;             // slice 0 position
    double thickness;      // slice thickness
    double dso;
    double dsd;

    HelicalInterpolationParam() {}
    HelicalInterpolationParam(unsigned int ns, unsigned int nt, unsigned int na, double ds, double dt,
                              double offset_s, double offset_t, double orbit_start, double orbit,
                              double couch_begin, double couch_mov, unsigned int view_per_rot,
                              unsigned int nz, double dz, double z0, double thickness, double dso,
                              double dsd)
        : ns(ns), nt(nt), na(na), ds(ds), dt(dt), offset_s(offset_s), offset_t(offset_t),
          orbit_start(orbit_start), orbit(orbit), couch_begin(couch_begin), couch_mov(couch_mov),
          view_per_rot(view_per_rot), nz(nz), dz(dz), z0(z0), thickness(thickness), dso(dso), dsd(dsd)
    {}
};

namespace detail {

inline ctr_helical_param helical_c(const HelicalInterpolationParam& p)
{
    ctr_helical_param c;
    c.ns = p.ns;
    c.nt = p.nt;
    c.na = p.na;
    c.ds = p.ds;
    c.dt = p.dt;
    c.offset_s = p.offset_s;
    c.offset_t = p.offset_t;
    c.orbit_start = p.orbit_start;
    c.orbit = p.orbit;
    c.couch_begin = p.couch_begin;
    c.couch_mov = p.couch_mov;
    c.view_per_rot = p.view_per_rot;
    c.nz = p.nz;
    c.dz = p.dz;
    c.z0 = p.z0;
    c.thickness = p.thickness;
    c.dso = p.dso;
    c.dsd = p.dsd;
    return c;
}

template <typename T>
bool helical_run(const HelicalInterpolationParam& param, int method, const T* in, T* out, cudaStream_t stream)
{
    const ctr_helical_param p = helical_c(param);
    const size_t bytes = ctr_helical_interpolation_table_bytes(&p);
    const size_t status_at = (bytes + 15) / 16 * 16;  // one status word per slice after the table
    const size_t status_bytes = sizeof(unsigned int) * p.nz;
    void* buf = nullptr;
    if (bytes == 0 || cudaMallocAsync(&buf, status_at + status_bytes, stream) != cudaSuccess) return false;
    unsigned int* status = reinterpret_cast<unsigned int*>(static_cast<char*>(buf) + status_at);
    std::vector<unsigned int> words(p.nz, 0u);
    int st = ctr_helical_interpolation_prep(&p, method, buf, stream);
    if (st == CTR_OK && cudaMemsetAsync(status, 0, status_bytes, stream) != cudaSuccess) st = CTR_ERR_CUDA;
    if (st == CTR_OK) {
        if (Precision<T>::is_double)
            st = method == CTR_HELICAL_360
                     ? ctr_helical_interpolation_360_f64(&p, reinterpret_cast<const double*>(in),
                                                         reinterpret_cast<double*>(out), buf, status, 1, stream)
                     : ctr_helical_interpolation_180_f64(&p, reinterpret_cast<const double*>(in),
                                                         reinterpret_cast<double*>(out), buf, status, 1, stream);
        else
            st = method == CTR_HELICAL_360
                     ? ctr_helical_interpolation_360_f32(&p, reinterpret_cast<const float*>(in),
                                                         reinterpret_cast<float*>(out), buf, status, 1, stream)
                     : ctr_helical_interpolation_180_f32(&p, reinterpret_cast<const float*>(in),
                                                         reinterpret_cast<float*>(out), buf, status, 1, stream);
    }
    if (st == CTR_OK &&
        cudaMemcpyAsync(words.data(), status, status_bytes, cudaMemcpyDeviceToHost, stream) != cudaSuccess)
        st = CTR_ERR_CUDA;
    cudaFreeAsync(buf, stream);
    const bool done = cudaStreamSynchronize(stream) == cudaSuccess;
    if (st != CTR_OK || !done) return false;
    // the reference processes slices in order and throws at the first problem
    for (unsigned int w : words) {
        if (w & CTR_HELICAL_BAD_TABLE) return false;
        if (w & CTR_HELICAL_NO_VIEWS) throw std::runtime_error("View not enough for this slice!");
        if (w & CTR_HELICAL_NO_ROWS) throw std::runtime_error("No row data available!");
    }
    return true;
}

}  // namespace detail

// reference include/helical_interpolation.h:66-82
template <typename T>
class HelicalInterpolation {
public:
    explicit HelicalInterpolation(const HelicalInterpolationParam& param) : param_(param) {}
    virtual ~HelicalInterpolation() {}
    // the reference's CPU implementation is not part of this library
    virtual bool calculate_on_cpu(const T*, T*) const { return false; }
    virtual bool calculate_on_gpu(const T* proj_in, T* proj_out, cudaStream_t stream) const = 0;

protected:
    HelicalInterpolationParam param_;
};

// 360LI, reference include/helical_interpolation.h:84-98
template <typename T>
class HelicalInterpolation360 : public HelicalInterpolation<T> {
public:
    explicit HelicalInterpolation360(const HelicalInterpolationParam& param) : HelicalInterpolation<T>(param) {}
    bool calculate_on_gpu(const T* proj_in, T* proj_out, cudaStream_t stream) const override
    {
        return detail::helical_run<T>(this->param_, CTR_HELICAL_360, proj_in, proj_out, stream);
    }
};

// 180LI, reference include/helical_interpolation.h:100-114
template <typename T>
class HelicalInterpolation180 : public HelicalInterpolation<T> {
public:
    explicit HelicalInterpolation180(const HelicalInterpolationParam& param) : HelicalInterpolation<T>(param) {}
    bool calculate_on_gpu(const T* proj_in, T* proj_out, cudaStream_t stream) const override
    {
        return detail::helical_run<T>(this->param_, CTR_HELICAL_180, proj_in, proj_out, stream);
    }
};

}  // namespace ct_recon

#endif
