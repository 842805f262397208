// C++ mirror of the reference's include/fp_par_2d.h (ray-driven parallel
// projection, its prep, grad prep and grad; ray casting and its prep;
// distance driven, its prep, grad prep and grad) over libctrecon_gb300.
#ifndef CT_RECON_GB300_FP_PAR_2D_H_
#define CT_RECON_GB300_FP_PAR_2D_H_

#include "ct_recon/bp_par_2d.h"

namespace ct_recon {

using ParallelProjection2DParam = ParallelBackprojection2DParam;

class ParallelProjection2DRayDrivenPrepare {
public:
    explicit ParallelProjection2DRayDrivenPrepare(const ParallelProjection2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelProjection2DRayDrivenPrepare() {}
    bool calculate_on_cpu(double*, double*, int*) const { return false; }
    // sincostbl double[na][2], beginoffset double[na][ns][2], usex int[na] (device)
    bool calculate_on_gpu(double* sincostbl, double* beginoffset, int* usex,
                          cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        return detail::finish(ctr_fp_par_2d_prep(&p, sincostbl, beginoffset, usex, stream), stream);
    }

protected:
    ParallelProjection2DParam param_;
};

class ParallelProjection2DRayDrivenGradPrep {
public:
    explicit ParallelProjection2DRayDrivenGradPrep(const ParallelProjection2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelProjection2DRayDrivenGradPrep() {}
    bool calculate_on_cpu(double*, double*, int*) const { return false; }
    // weights double[na], pos double[na][nx][2], usex int[na] (device)
    bool calculate_on_gpu(double* weights, double* pos, int* usex, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        return detail::finish(ctr_fp_par_2d_grad_prep(&p, weights, pos, usex, stream), stream);
    }

protected:
    ParallelProjection2DParam param_;
};

template <typename T>
class ParallelProjection2DRayDriven {
public:
    explicit ParallelProjection2DRayDriven(const ParallelProjection2DParam& param) : param_(param) {}
    virtual ~ParallelProjection2DRayDriven() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const int*) const
    {
        return false;
    }
    bool calculate_on_gpu(const T* img, T* proj, const double* sincostbl,
                          const double* beginoffset, const int* usex, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_fp_par_2d_f64(&p, reinterpret_cast<const double*>(img),
                                               reinterpret_cast<double*>(proj), sincostbl,
                                               beginoffset, usex, 1, stream)
                           : ctr_fp_par_2d_f32(&p, reinterpret_cast<const float*>(img),
                                               reinterpret_cast<float*>(proj), sincostbl,
                                               beginoffset, usex, 1, stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelProjection2DParam param_;
};

template <typename T>
class ParallelProjection2DRayDrivenGrad {
public:
    explicit ParallelProjection2DRayDrivenGrad(const ParallelProjection2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelProjection2DRayDrivenGrad() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const int*) const
    {
        return false;
    }
    bool calculate_on_gpu(const T* proj, T* img, const double* weights, const double* pos,
                          const int* usex, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_fp_par_2d_grad_f64(&p, reinterpret_cast<const double*>(proj),
                                                    reinterpret_cast<double*>(img), weights, pos,
                                                    usex, 1, stream)
                           : ctr_fp_par_2d_grad_f32(&p, reinterpret_cast<const float*>(proj),
                                                    reinterpret_cast<float*>(img), weights, pos,
                                                    usex, 1, stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelProjection2DParam param_;
};

// Ray casting (reference include/fp_par_2d.h:155-203): samples every step_size
// pixels inside the FoV circle of radius fov; no gradient, as in the reference.
class ParallelProjection2DRayCastingPrepare {
public:
    explicit ParallelProjection2DRayCastingPrepare(const ParallelProjection2DParam& param,
                                                   const double step_size = 0.125)
        : param_(param), step_size_(step_size)
    {}
    virtual ~ParallelProjection2DRayCastingPrepare() {}
    bool calculate_on_cpu(double*, double*, int*) const { return false; }
    // sincostbl double[na][2], begins double[na][ns][2], nsteps int[na][ns] (device)
    bool calculate_on_gpu(double* sincostbl, double* begins, int* nsteps, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        return detail::finish(ctr_fp_par_2d_cast_prep(&p, step_size_, sincostbl, begins, nsteps, stream),
                              stream);
    }

protected:
    ParallelProjection2DParam param_;
    double step_size_;
};

template <typename T>
class ParallelProjection2DRayCasting {
public:
    explicit ParallelProjection2DRayCasting(const ParallelProjection2DParam& param,
                                            const double step_size = 0.125)
        : param_(param), step_size_(step_size)
    {}
    virtual ~ParallelProjection2DRayCasting() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const int*) const
    {
        return false;
    }
    bool calculate_on_gpu(const T* img, T* proj, const double* sincostbl, const double* begins,
                          const int* nsteps, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_fp_par_2d_cast_f64(&p, step_size_, reinterpret_cast<const double*>(img),
                                                    reinterpret_cast<double*>(proj), sincostbl, begins,
                                                    nsteps, 1, stream)
                           : ctr_fp_par_2d_cast_f32(&p, step_size_, reinterpret_cast<const float*>(img),
                                                    reinterpret_cast<float*>(proj), sincostbl, begins,
                                                    nsteps, 1, stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelProjection2DParam param_;
    double step_size_;
};

// Distance driven (reference include/fp_par_2d.h:283-352); the grad is the
// reference's distance-driven grad.
class ParallelProjection2DDisDrivenPrep {
public:
    explicit ParallelProjection2DDisDrivenPrep(const ParallelProjection2DParam& param) : param_(param) {}
    virtual ~ParallelProjection2DDisDrivenPrep() {}
    bool calculate_on_cpu(double*, double*, int*) const { return false; }
    // sincostbl double[na][2], beginoffset double[na][ns][3], usex int[na] (device)
    bool calculate_on_gpu(double* sincostbl, double* beginoffset, int* usex, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        return detail::finish(ctr_fp_par_2d_dd_prep(&p, sincostbl, beginoffset, usex, stream), stream);
    }

protected:
    ParallelProjection2DParam param_;
};

class ParallelProjection2DDisDrivenGradPrep {
public:
    explicit ParallelProjection2DDisDrivenGradPrep(const ParallelProjection2DParam& param)
        : param_(param)
    {}
    virtual ~ParallelProjection2DDisDrivenGradPrep() {}
    bool calculate_on_cpu(double*, double*, int*) const { return false; }
    // weights double[na], pos double[na][nx][2], usex int[na] (device)
    bool calculate_on_gpu(double* weights, double* pos, int* usex, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        return detail::finish(ctr_fp_par_2d_dd_grad_prep(&p, weights, pos, usex, stream), stream);
    }

protected:
    ParallelProjection2DParam param_;
};

template <typename T>
class ParallelProjection2DDisDriven {
public:
    explicit ParallelProjection2DDisDriven(const ParallelProjection2DParam& param) : param_(param) {}
    virtual ~ParallelProjection2DDisDriven() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const int*) const { return false; }
    bool calculate_on_gpu(const T* img, T* proj, const double* sincostbl, const double* beginoffset,
                          const int* usex, cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_fp_par_2d_dd_f64(&p, reinterpret_cast<const double*>(img),
                                                  reinterpret_cast<double*>(proj), sincostbl, beginoffset,
                                                  usex, 1, stream)
                           : ctr_fp_par_2d_dd_f32(&p, reinterpret_cast<const float*>(img),
                                                  reinterpret_cast<float*>(proj), sincostbl, beginoffset,
                                                  usex, 1, stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelProjection2DParam param_;
};

template <typename T>
class ParallelProjection2DDisDrivenGrad {
public:
    explicit ParallelProjection2DDisDrivenGrad(const ParallelProjection2DParam& param) : param_(param) {}
    virtual ~ParallelProjection2DDisDrivenGrad() {}
    bool calculate_on_cpu(const T*, T*, const double*, const double*, const int*) const { return false; }
    bool calculate_on_gpu(const T* proj, T* img, const double* weights, const double* pos, const int* usex,
                          cudaStream_t stream) const
    {
        const ctr_par_param p = param_.c();
        const int st = detail::Precision<T>::is_double
                           ? ctr_fp_par_2d_dd_grad_f64(&p, reinterpret_cast<const double*>(proj),
                                                       reinterpret_cast<double*>(img), weights, pos, usex, 1,
                                                       stream)
                           : ctr_fp_par_2d_dd_grad_f32(&p, reinterpret_cast<const float*>(proj),
                                                       reinterpret_cast<float*>(img), weights, pos, usex, 1,
                                                       stream);
        return detail::finish(st, stream);
    }

protected:
    ParallelProjection2DParam param_;
};

}  // namespace ct_recon
#endif
