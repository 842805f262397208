// C++ mirror of the reference's include/filter.h (FilterParam, RampFilterPrep,
// RampFilter<T>, RampFilterGrad<T>) over libctrecon_gb300.
#ifndef CT_RECON_GB300_FILTER_H_
#define CT_RECON_GB300_FILTER_H_

#include "ct_recon/common.h"

namespace ct_recon {

struct FilterParam {
    unsigned int ns, nrow;
    double ds, dsd;
    int type;    // 0 "par", 1 "fan", 2 "flat"
    int window;  // unused
    FilterParam() {}
    FilterParam(unsigned int ns, unsigned int nrow, double ds, double dsd = -1, int type = 0,
                int window = 0)
        : ns(ns), nrow(nrow), ds(ds), dsd(dsd), type(type), window(window)
    {}
    ctr_filter_param c() const { return {ns, nrow, ds, dsd, type, window}; }
};

class RampFilterPrep {
public:
    explicit RampFilterPrep(const FilterParam& param) : param_(param) {}
    bool calculate_on_cpu(double*) const { return false; }
    // filter: device double[2*ns+1]
    bool calculate_on_gpu(double* filter, cudaStream_t stream) const
    {
        const ctr_filter_param p = param_.c();
        return detail::finish(ctr_ramp_filter_prep(&p, filter, stream), stream);
    }

private:
    FilterParam param_;
};

template <typename T, bool kGrad>
class RampFilterBase {
public:
    explicit RampFilterBase(const FilterParam& param) : param_(param) {}
    bool calculate_on_cpu(const T*, const double*, T*) const { return false; }
    bool calculate_on_gpu(const T* in, const double* filter, T* out, cudaStream_t stream) const
    {
        const ctr_filter_param p = param_.c();
        int st;
        if (detail::Precision<T>::is_double)
            st = (kGrad ? ctr_ramp_filter_grad_f64 : ctr_ramp_filter_f64)(
                &p, reinterpret_cast<const double*>(in), filter, reinterpret_cast<double*>(out), 1,
                stream);
        else
            st = (kGrad ? ctr_ramp_filter_grad_f32 : ctr_ramp_filter_f32)(
                &p, reinterpret_cast<const float*>(in), filter, reinterpret_cast<float*>(out), 1,
                stream);
        return detail::finish(st, stream);
    }

private:
    FilterParam param_;
};

template <typename T>
class RampFilter : public RampFilterBase<T, false> {
public:
    using RampFilterBase<T, false>::RampFilterBase;
};

template <typename T>
class RampFilterGrad : public RampFilterBase<T, true> {
public:
    using RampFilterBase<T, true>::RampFilterBase;
};

}  // namespace ct_recon
#endif
