// C++ mirror of the reference's include/fan_weighting.h (FanWeightingParam,
// FanWeighting<T>, FanWeightingGrad<T>) over libctrecon_gb300.
#ifndef CT_RECON_GB300_FAN_WEIGHTING_H_
#define CT_RECON_GB300_FAN_WEIGHTING_H_

#include "ct_recon/common.h"

namespace ct_recon {

struct FanWeightingParam {
    unsigned int ns, nrow;
    double ds, offset, dso, dsd;
    int type;  // 1 "fan", 2 "flat"
    FanWeightingParam() {}
    FanWeightingParam(unsigned int ns, unsigned int nrow, double ds, double offset = 0,
                      double dso = -1, double dsd = -1, int type = 1)
        : ns(ns), nrow(nrow), ds(ds), offset(offset), dso(dso), dsd(dsd), type(type)
    {}
    ctr_fan_weighting_param c() const { return {ns, nrow, ds, offset, dso, dsd, type}; }
};

template <typename T>
class FanWeighting {
public:
    explicit FanWeighting(const FanWeightingParam& param) : param_(param) {}
    bool calculate_on_cpu(const T*, T*) const { return false; }
    bool calculate_on_gpu(const T* in, T* out, cudaStream_t stream) const
    {
        const ctr_fan_weighting_param p = param_.c();
        if (detail::Precision<T>::is_double)
            return detail::finish(ctr_fan_weighting_f64(&p, reinterpret_cast<const double*>(in),
                                                        reinterpret_cast<double*>(out), 1, stream),
                                  stream);
        return detail::finish(ctr_fan_weighting_f32(&p, reinterpret_cast<const float*>(in),
                                                    reinterpret_cast<float*>(out), 1, stream),
                              stream);
    }

private:
    FanWeightingParam param_;
};

template <typename T>
class FanWeightingGrad {
public:
    explicit FanWeightingGrad(const FanWeightingParam& param) : param_(param) {}
    bool calculate_on_cpu(const T*, T*) const { return false; }
    bool calculate_on_gpu(const T* in, T* out, cudaStream_t stream) const
    {
        const ctr_fan_weighting_param p = param_.c();
        if (detail::Precision<T>::is_double)
            return detail::finish(ctr_fan_weighting_grad_f64(&p, reinterpret_cast<const double*>(in),
                                                             reinterpret_cast<double*>(out), 1, stream),
                                  stream);
        return detail::finish(ctr_fan_weighting_grad_f32(&p, reinterpret_cast<const float*>(in),
                                                         reinterpret_cast<float*>(out), 1, stream),
                              stream);
    }

private:
    FanWeightingParam param_;
};

}  // namespace ct_recon
#endif
