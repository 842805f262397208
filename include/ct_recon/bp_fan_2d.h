// C++ mirror of the reference's include/bp_fan_2d.h over libctrecon_gb300:
// FanBackprojection2DParam, the abstract Prepare / Backprojection / GradPrep /
// Grad classes and their pixel-driven implementations.
#ifndef CT_RECON_GB300_BP_FAN_2D_H_
#define CT_RECON_GB300_BP_FAN_2D_H_

#include "ct_recon/common.h"

namespace ct_recon {

struct FanBackprojection2DParam {
    unsigned int ns, na;
    double ds, orbit, offset_s, orbit_start;
    unsigned int nx, ny;
    double dx, dy, offset_x, offset_y, dso, dsd, fov;
    FanBackprojection2DParam() {}
    FanBackprojection2DParam(unsigned int ns, unsigned int na, double ds, double orbit,
                             double offset_s, double orbit_start, unsigned int nx, unsigned int ny,
                             double dx, double dy, double offset_x, double offset_y, double dso,
                             double dsd, double fov)
        : ns(ns), na(na), ds(ds), orbit(orbit), offset_s(offset_s), orbit_start(orbit_start),
          nx(nx), ny(ny), dx(dx), dy(dy), offset_x(offset_x), offset_y(offset_y), dso(dso),
          dsd(dsd), fov(fov)
    {}
    ctr_fan_bp_param c() const
    {
        return {ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, offset_x, offset_y,
                dso, dsd, fov};
    }
};

class FanBackprojection2DPrepare {
public:
    explicit FanBackprojection2DPrepare(const FanBackprojection2DParam& param) : param_(param) {}
    virtual ~FanBackprojection2DPrepare() {}
    virtual bool calculate_on_cpu(double*, double*, double*) const = 0;
    virtual bool calculate_on_gpu(double*, double*, double*, cudaStream_t) const = 0;

protected:
    FanBackprojection2DParam param_;
};

template <typename T>
class FanBackprojection2D {
public:
    explicit FanBackprojection2D(const FanBackprojection2DParam& param) : param_(param) {}
    virtual ~FanBackprojection2D() {}
    virtual bool calculate_on_cpu(const T*, T*, const double*, const double*, const double*) const = 0;
    virtual bool calculate_on_gpu(const T*, T*, const double*, const double*, const double*,
                                  cudaStream_t) const = 0;

protected:
    FanBackprojection2DParam param_;
};

class FanBackprojection2DGradPrep : public FanBackprojection2DPrepare {
public:
    using FanBackprojection2DPrepare::FanBackprojection2DPrepare;
};

template <typename T>
class FanBackprojection2DGrad : public FanBackprojection2D<T> {
public:
    using FanBackprojection2D<T>::FanBackprojection2D;
};

class FanBackprojection2DPixDrivenPrep : public FanBackprojection2DPrepare {
public:
    using FanBackprojection2DPrepare::FanBackprojection2DPrepare;
    bool calculate_on_cpu(double*, double*, double*) const override { return false; }
    // xpos double[nx], ypos double[ny], sincostbl double[2*na] (device)
    bool calculate_on_gpu(double* xpos, double* ypos, double* sincostbl,
                          cudaStream_t stream) const override
    {
        const ctr_fan_bp_param p = param_.c();
        return detail::finish(ctr_bp_fan_2d_prep(&p, xpos, ypos, sincostbl, stream), stream);
    }
};

class FanBackprojection2DPixDrivenGradPrep : public FanBackprojection2DGradPrep {
public:
    using FanBackprojection2DGradPrep::FanBackprojection2DGradPrep;
    bool calculate_on_cpu(double*, double*, double*) const override { return false; }
    bool calculate_on_gpu(double* xpos, double* ypos, double* sincostbl,
                          cudaStream_t stream) const override
    {
        const ctr_fan_bp_param p = param_.c();
        return detail::finish(ctr_bp_fan_2d_prep(&p, xpos, ypos, sincostbl, stream), stream);
    }
};

template <typename T>
class FanBackprojection2DPixDriven : public FanBackprojection2D<T> {
public:
    using FanBackprojection2D<T>::FanBackprojection2D;
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const double*) const override
    {
        return false;
    }
    bool calculate_on_gpu(const T* proj, T* img, const double* xpos, const double* ypos,
                          const double* sincostbl, cudaStream_t stream) const override
    {
        const ctr_fan_bp_param p = this->param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_bp_fan_2d_f64(&p, reinterpret_cast<const double*>(proj),
                                               reinterpret_cast<double*>(img), xpos, ypos,
                                               sincostbl, 1, stream)
                           : ctr_bp_fan_2d_f32(&p, reinterpret_cast<const float*>(proj),
                                               reinterpret_cast<float*>(img), xpos, ypos,
                                               sincostbl, 1, stream);
        return detail::finish(st, stream);
    }
};

template <typename T>
class FanBackprojection2DPixDrivenGrad : public FanBackprojection2DGrad<T> {
public:
    using FanBackprojection2DGrad<T>::FanBackprojection2DGrad;
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const double*) const override
    {
        return false;
    }
    // img [ny][nx] -> grad [na][ns]
    bool calculate_on_gpu(const T* img, T* grad, const double* xpos, const double* ypos,
                          const double* sincostbl, cudaStream_t stream) const override
    {
        const ctr_fan_bp_param p = this->param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_bp_fan_2d_grad_f64(&p, reinterpret_cast<const double*>(img),
                                                    reinterpret_cast<double*>(grad), xpos, ypos,
                                                    sincostbl, 1, stream)
                           : ctr_bp_fan_2d_grad_f32(&p, reinterpret_cast<const float*>(img),
                                                    reinterpret_cast<float*>(grad), xpos, ypos,
                                                    sincostbl, 1, stream);
        return detail::finish(st, stream);
    }
};

}  // namespace ct_recon
#endif
