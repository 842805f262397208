// C++ mirror of the reference's include/bp_fan_2d_angle.h over libctrecon_gb300
// (explicit angle list, no output scale).  The grad is the exact adjoint of the
// backprojection (the reference's grad is not well defined).
#ifndef CT_RECON_GB300_BP_FAN_2D_ANGLE_H_
#define CT_RECON_GB300_BP_FAN_2D_ANGLE_H_

#include "ct_recon/common.h"

namespace ct_recon {

struct FanBackprojection2DAngleParam {
    unsigned int ns, na;
    double ds, offset_s;
    unsigned int nx, ny;
    double dx, dy, offset_x, offset_y, dso, dsd, fov;
    FanBackprojection2DAngleParam() {}
    FanBackprojection2DAngleParam(unsigned int ns, unsigned int na, double ds, double offset_s,
                                  unsigned int nx, unsigned int ny, double dx, double dy,
                                  double offset_x, double offset_y, double dso, double dsd,
                                  double fov)
        : ns(ns), na(na), ds(ds), offset_s(offset_s), nx(nx), ny(ny), dx(dx), dy(dy),
          offset_x(offset_x), offset_y(offset_y), dso(dso), dsd(dsd), fov(fov)
    {}
    ctr_fan_bp_angle_param c() const
    {
        return {ns, na, ds, offset_s, nx, ny, dx, dy, offset_x, offset_y, dso, dsd, fov};
    }
};

class FanBackprojection2DAnglePixDrivenPrep {
public:
    explicit FanBackprojection2DAnglePixDrivenPrep(const FanBackprojection2DAngleParam& param)
        : param_(param)
    {}
    virtual ~FanBackprojection2DAnglePixDrivenPrep() {}
    bool calculate_on_cpu(const double*, double*, double*, double*) const { return false; }
    // angles: device double[na]
    bool calculate_on_gpu(const double* angles, double* xpos, double* ypos, double* sincostbl,
                          cudaStream_t stream) const
    {
        const ctr_fan_bp_angle_param p = param_.c();
        return detail::finish(ctr_bp_fan_2d_angle_prep(&p, angles, xpos, ypos, sincostbl, stream),
                              stream);
    }

protected:
    FanBackprojection2DAngleParam param_;
};

using FanBackprojection2DAnglePixDrivenGradPrep = FanBackprojection2DAnglePixDrivenPrep;

template <typename T, bool kGrad>
class FanBackprojection2DAngleBase {
public:
    explicit FanBackprojection2DAngleBase(const FanBackprojection2DAngleParam& param)
        : param_(param)
    {}
    virtual ~FanBackprojection2DAngleBase() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const double*) const
    {
        return false;
    }
    bool calculate_on_gpu(const T* in, T* out, const double* xpos, const double* ypos,
                          const double* sincostbl, cudaStream_t stream) const
    {
        const ctr_fan_bp_angle_param p = param_.c();
        int st;
        if (detail::Precision<T>::is_double)
            st = (kGrad ? ctr_bp_fan_2d_angle_grad_f64 : ctr_bp_fan_2d_angle_f64)(
                &p, reinterpret_cast<const double*>(in), reinterpret_cast<double*>(out), xpos,
                ypos, sincostbl, 1, stream);
        else
            st = (kGrad ? ctr_bp_fan_2d_angle_grad_f32 : ctr_bp_fan_2d_angle_f32)(
                &p, reinterpret_cast<const float*>(in), reinterpret_cast<float*>(out), xpos,
                ypos, sincostbl, 1, stream);
        return detail::finish(st, stream);
    }

protected:
    FanBackprojection2DAngleParam param_;
};

template <typename T>
class FanBackprojection2DAnglePixDriven : public FanBackprojection2DAngleBase<T, false> {
public:
    using FanBackprojection2DAngleBase<T, false>::FanBackprojection2DAngleBase;
};

template <typename T>
class FanBackprojection2DAnglePixDrivenGrad : public FanBackprojection2DAngleBase<T, true> {
public:
    using FanBackprojection2DAngleBase<T, true>::FanBackprojection2DAngleBase;
};

}  // namespace ct_recon
#endif
