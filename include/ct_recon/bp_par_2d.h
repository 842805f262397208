// C++ mirror of the reference's include/bp_par_2d.h (pixel-driven parallel
// backprojection) and include/bp_par_2d_sv.h (single view) over libctrecon_gb300.
// The grad takes the forward's tables and is the exact adjoint of the forward
// (the reference's grad pair is not well defined).
#ifndef CT_RECON_GB300_BP_PAR_2D_H_
#define CT_RECON_GB300_BP_PAR_2D_H_

#include "ct_recon/common.h"

namespace ct_recon {

struct ParallelBackprojection2DParam {
    unsigned int ns, na;
    double ds, orbit, offset_s, orbit_start;
    unsigned int nx, ny;
    double dx, dy, offset_x, offset_y, fov;
    ParallelBackprojection2DParam() {}
    ParallelBackprojection2DParam(unsigned int ns, unsigned int na, double ds, double orbit,
                                  double offset_s, double orbit_start, unsigned int nx,
                                  unsigned int ny, double dx, double dy, double offset_x,
                                  double offset_y, double fov)
        : ns(ns), na(na), ds(ds), orbit(orbit), offset_s(offset_s), orbit_start(orbit_start),
          nx(nx), ny(ny), dx(dx), dy(dy), offset_x(offset_x), offset_y(offset_y), fov(fov)
    {}
    ctr_par_param c() const
    {
        return {ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x, offset_y, fov};
    }
};
using ParallelSingleViewBp2DParam = ParallelBackprojection2DParam;

class ParallelBackprojection2DPixDrivenPrep {
public:
    explicit ParallelBackprojection2DPixDrivenPrep(const ParallelBackprojection2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelBackprojection2DPixDrivenPrep() {}
    bool calculate_on_cpu(double*, double*, int*) const { return false; }
    // xcos double[nx][na], ysin double[ny][na] (device); buffer unused
    bool calculate_on_gpu(double* xcos, double* ysin, int* buffer, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        return detail::finish(ctr_bp_par_2d_prep(&p, xcos, ysin, buffer, stream), stream);
    }

protected:
    ParallelBackprojection2DParam param_;
};
using ParallelSingleViewBp2DPixDrivenPrep = ParallelBackprojection2DPixDrivenPrep;

template <typename T>
class ParallelBackprojection2DPixDriven {
public:
    explicit ParallelBackprojection2DPixDriven(const ParallelBackprojection2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelBackprojection2DPixDriven() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const int*) const
    {
        return false;
    }
    bool calculate_on_gpu(const T* proj, T* img, const double* xcos, const double* ysin,
                          const int* buffer, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_bp_par_2d_f64(&p, reinterpret_cast<const double*>(proj),
                                               reinterpret_cast<double*>(img), xcos, ysin, buffer,
                                               1, stream)
                           : ctr_bp_par_2d_f32(&p, reinterpret_cast<const float*>(proj),
                                               reinterpret_cast<float*>(img), xcos, ysin, buffer,
                                               1, stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelBackprojection2DParam param_;
};

template <typename T>
class ParallelBackprojection2DPixDrivenGrad {
public:
    explicit ParallelBackprojection2DPixDrivenGrad(const ParallelBackprojection2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelBackprojection2DPixDrivenGrad() {}
    // img [ny][nx] -> grad [na][ns]; xcos/ysin are the forward's tables
    bool calculate_on_gpu(const T* img, T* grad, const double* xcos, const double* ysin,
                          cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_bp_par_2d_grad_f64(&p, reinterpret_cast<const double*>(img),
                                                    reinterpret_cast<double*>(grad), xcos, ysin, 1,
                                                    stream)
                           : ctr_bp_par_2d_grad_f32(&p, reinterpret_cast<const float*>(img),
                                                    reinterpret_cast<float*>(grad), xcos, ysin, 1,
                                                    stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelBackprojection2DParam param_;
};

template <typename T>
class ParallelSingleViewBp2DPixDriven {
public:
    explicit ParallelSingleViewBp2DPixDriven(const ParallelSingleViewBp2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelSingleViewBp2DPixDriven() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const int*) const
    {
        return false;
    }
    // proj [na][ns] -> img [ny][nx][na]
    bool calculate_on_gpu(const T* proj, T* img, const double* xcos, const double* ysin,
                          const int* buffer, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_bp_par_2d_sv_f64(&p, reinterpret_cast<const double*>(proj),
                                                  reinterpret_cast<double*>(img), xcos, ysin,
                                                  buffer, 1, stream)
                           : ctr_bp_par_2d_sv_f32(&p, reinterpret_cast<const float*>(proj),
                                                  reinterpret_cast<float*>(img), xcos, ysin,
                                                  buffer, 1, stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelSingleViewBp2DParam param_;
};

}  // namespace ct_recon
#endif
