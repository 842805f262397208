// C entry points over the reference's own CPU classes -- TEST INFRASTRUCTURE.
//
// Compiled (oracle/Makefile, target "ref") together with the reference's
// src/*.cc straight from the reference checkout, into oracle/_ref/.  It gives
// tests/golden/make_golden.py and the pin tests the reference's own outputs
// through the same signatures as ctr_oracle.h (prefix ref_ instead of orc_).
// Only methods whose reference code is well defined are exposed: the
// parallel-BP grad (src/bp_par_2d.cc:145-199, uninitialised pointers) and the
// fan-angle grad (src/bp_fan_2d_angle.cc:124-169, uninitialised ypos) are not.
#include <stdexcept>
#include <string>
#include <vector>

#include "include/bp_fan_2d.h"
#include "include/bp_fan_2d_angle.h"
#include "include/bp_par_2d.h"
#include "include/bp_par_2d_sv.h"
#include "include/fan_weighting.h"
#include "include/filter.h"
#include "include/fp_par_2d.h"
#include "include/helical_interpolation.h"

#include "ctr_oracle.h"

using namespace ct_recon;

namespace {

HelicalInterpolationParam heli_param(const orc_heli* h)
{
    return HelicalInterpolationParam(h->ns, h->nt, h->na, h->ds, h->dt, h->offset_s, h->offset_t,
                                     h->orbit_start, h->orbit, h->couch_begin, h->couch_mov,
                                     h->view_per_rot, h->nz, h->dz, h->z0, h->thickness, h->dso,
                                     h->dsd);
}

int heli_error(const std::runtime_error& e)
{
    return std::string(e.what()).find("View") != std::string::npos ? ORC_HELI_ERR_VIEWS
                                                                    : ORC_HELI_ERR_ROWS;
}

FanBackprojection2DParam fan_param(const orc_geom* g)
{
    return FanBackprojection2DParam(g->ns, g->na, g->ds, g->orbit, g->offset_s, g->orbit_start,
                                    g->nx, g->ny, g->dx, g->dy, g->offset_x, g->offset_y,
                                    g->dso, g->dsd, g->fov);
}

FanBackprojection2DAngleParam angle_param(const orc_geom* g)
{
    return FanBackprojection2DAngleParam(g->ns, g->na, g->ds, g->offset_s, g->nx, g->ny, g->dx,
                                         g->dy, g->offset_x, g->offset_y, g->dso, g->dsd,
                                         g->fov);
}

ParallelBackprojection2DParam par_param(const orc_geom* g)
{
    return ParallelBackprojection2DParam(g->ns, g->na, g->ds, g->orbit, g->offset_s,
                                         g->orbit_start, g->nx, g->ny, g->dx, g->dy,
                                         g->offset_x, g->offset_y, g->fov);
}

ParallelSingleViewBp2DParam sv_param(const orc_geom* g)
{
    return ParallelSingleViewBp2DParam(g->ns, g->na, g->ds, g->orbit, g->offset_s,
                                       g->orbit_start, g->nx, g->ny, g->dx, g->dy, g->offset_x,
                                       g->offset_y, g->fov);
}

ParallelProjection2DParam fp_param(const orc_geom* g)
{
    return ParallelProjection2DParam(g->ns, g->na, g->ds, g->orbit, g->offset_s, g->orbit_start,
                                     g->nx, g->ny, g->dx, g->dy, g->offset_x, g->offset_y,
                                     g->fov);
}

}  // namespace

#define REF_T(T, SFX)                                                                          \
    extern "C" int ref_fan_weighting_##SFX(unsigned ns, unsigned nrow, double ds,              \
                                           double offset, double dso, double dsd, int type,    \
                                           const T* in, T* out)                                \
    {                                                                                          \
        return FanWeighting<T>(FanWeightingParam(ns, nrow, ds, offset, dso, dsd, type))        \
            .calculate_on_cpu(in, out);                                                        \
    }                                                                                          \
    extern "C" int ref_fan_weighting_grad_##SFX(unsigned ns, unsigned nrow, double ds,         \
                                                double offset, double dso, double dsd,         \
                                                int type, const T* in, T* out)                 \
    {                                                                                          \
        return FanWeightingGrad<T>(FanWeightingParam(ns, nrow, ds, offset, dso, dsd, type))    \
            .calculate_on_cpu(in, out);                                                        \
    }                                                                                          \
    extern "C" int ref_ramp_filter_##SFX(unsigned ns, unsigned nrow, double ds, const T* in,   \
                                         const double* filter, T* out)                         \
    {                                                                                          \
        return RampFilter<T>(FilterParam(ns, nrow, ds)).calculate_on_cpu(in, filter, out);     \
    }                                                                                          \
    extern "C" int ref_ramp_filter_grad_##SFX(unsigned ns, unsigned nrow, double ds,           \
                                              const T* in, const double* filter, T* out)       \
    {                                                                                          \
        return RampFilterGrad<T>(FilterParam(ns, nrow, ds)).calculate_on_cpu(in, filter, out); \
    }                                                                                          \
    extern "C" int ref_bp_fan_2d_##SFX(const orc_geom* g, const T* proj, T* img,               \
                                       const double* xpos, const double* ypos,                 \
                                       const double* sc)                                       \
    {                                                                                          \
        return FanBackprojection2DPixDriven<T>(fan_param(g))                                   \
            .calculate_on_cpu(proj, img, xpos, ypos, sc);                                      \
    }                                                                                          \
    extern "C" int ref_bp_fan_2d_grad_##SFX(const orc_geom* g, const T* img, T* grad,          \
                                            const double* xpos, const double* ypos,            \
                                            const double* sc)                                  \
    {                                                                                          \
        return FanBackprojection2DPixDrivenGrad<T>(fan_param(g))                               \
            .calculate_on_cpu(img, grad, xpos, ypos, sc);                                      \
    }                                                                                          \
    extern "C" int ref_bp_fan_2d_angle_##SFX(const orc_geom* g, const T* proj, T* img,         \
                                             const double* xpos, const double* ypos,           \
                                             const double* sc)                                 \
    {                                                                                          \
        return FanBackprojection2DAnglePixDriven<T>(angle_param(g))                            \
            .calculate_on_cpu(proj, img, xpos, ypos, sc);                                      \
    }                                                                                          \
    extern "C" int ref_bp_par_2d_##SFX(const orc_geom* g, const T* proj, T* img,               \
                                       const double* xcos, const double* ysin)                 \
    {                                                                                          \
        return ParallelBackprojection2DPixDriven<T>(par_param(g))                              \
            .calculate_on_cpu(proj, img, xcos, ysin, nullptr);                                 \
    }                                                                                          \
    extern "C" int ref_bp_par_2d_sv_##SFX(const orc_geom* g, const T* proj, T* img,            \
                                          const double* xcos, const double* ysin)              \
    {                                                                                          \
        return ParallelSingleViewBp2DPixDriven<T>(sv_param(g))                                 \
            .calculate_on_cpu(proj, img, xcos, ysin, nullptr);                                 \
    }                                                                                          \
    extern "C" int ref_fp_par_2d_##SFX(const orc_geom* g, const T* img, T* proj,               \
                                       const double* sc, const double* bo, const int* usex)    \
    {                                                                                          \
        return ParallelProjection2DRayDriven<T>(fp_param(g))                                   \
            .calculate_on_cpu(img, proj, sc, bo, usex);                                        \
    }                                                                                          \
    extern "C" int ref_fp_par_2d_grad_##SFX(const orc_geom* g, const T* proj, T* img,          \
                                            const double* weights, const double* pos,          \
                                            const int* usex)                                   \
    {                                                                                          \
        return ParallelProjection2DRayDrivenGrad<T>(fp_param(g))                               \
            .calculate_on_cpu(proj, img, weights, pos, usex);                                  \
    }

#define REF_CAST(T, SFX)                                                                       \
    extern "C" int ref_fp_par_2d_cast_##SFX(const orc_geom* g, double step_size, const T* img,  \
                                            T* proj, const double* sc, const double* begins,    \
                                            const int* nsteps)                                  \
    {                                                                                          \
        return ParallelProjection2DRayCasting<T>(fp_param(g), step_size)                       \
            .calculate_on_cpu(img, proj, sc, begins, nsteps);                                  \
    }

#define REF_DD(T, SFX)                                                                         \
    extern "C" int ref_fp_par_2d_dd_##SFX(const orc_geom* g, const T* img, T* proj,            \
                                          const double* sc, const double* bo, const int* usex) \
    {                                                                                          \
        return ParallelProjection2DDisDriven<T>(fp_param(g))                                   \
            .calculate_on_cpu(img, proj, sc, bo, usex);                                        \
    }                                                                                          \
    extern "C" int ref_fp_par_2d_dd_grad_##SFX(const orc_geom* g, const T* proj, T* img,       \
                                               const double* w, const double* pos,             \
                                               const int* usex)                                \
    {                                                                                          \
        return ParallelProjection2DDisDrivenGrad<T>(fp_param(g))                               \
            .calculate_on_cpu(proj, img, w, pos, usex);                                        \
    }

// Helical rebinning: the reference throws std::runtime_error; the message
// maps to the oracle's codes (-1 "View not enough ...", -2 "No row data ...").
#define REF_HELI(T, SFX)                                                                       \
    extern "C" int ref_helical_360_##SFX(const orc_heli* h, const T* in, T* out)               \
    {                                                                                          \
        try {                                                                                  \
            return HelicalInterpolation360<T>(heli_param(h)).calculate_on_cpu(in, out);        \
        } catch (const std::runtime_error& e) {                                                \
            return heli_error(e);                                                              \
        }                                                                                      \
    }                                                                                          \
    extern "C" int ref_helical_180_##SFX(const orc_heli* h, const T* in, T* out)               \
    {                                                                                          \
        try {                                                                                  \
            return HelicalInterpolation180<T>(heli_param(h)).calculate_on_cpu(in, out);        \
        } catch (const std::runtime_error& e) {                                                \
            return heli_error(e);                                                              \
        }                                                                                      \
    }

REF_T(float, f32)
REF_T(double, f64)
REF_HELI(float, f32)
REF_HELI(double, f64)
REF_CAST(float, f32)
REF_CAST(double, f64)
REF_DD(float, f32)
REF_DD(double, f64)

extern "C" int ref_fp_par_2d_dd_prep(const orc_geom* g, double* sc, double* bo, int* usex)
{
    return ParallelProjection2DDisDrivenPrep(fp_param(g)).calculate_on_cpu(sc, bo, usex);
}

extern "C" int ref_fp_par_2d_dd_grad_prep(const orc_geom* g, double* w, double* pos, int* usex)
{
    return ParallelProjection2DDisDrivenGradPrep(fp_param(g)).calculate_on_cpu(w, pos, usex);
}

extern "C" int ref_fp_par_2d_cast_prep(const orc_geom* g, double step_size, double* sc,
                                       double* begins, int* nsteps)
{
    return ParallelProjection2DRayCastingPrepare(fp_param(g), step_size)
        .calculate_on_cpu(sc, begins, nsteps);
}

extern "C" int ref_ramp_filter_prep(unsigned ns, double ds, double dsd, int type,
                                    double* filter)
{
    return RampFilterPrep(FilterParam(ns, 1, ds, dsd, type)).calculate_on_cpu(filter);
}

extern "C" int ref_bp_fan_2d_prep(const orc_geom* g, double* xpos, double* ypos, double* sc)
{
    return FanBackprojection2DPixDrivenPrep(fan_param(g)).calculate_on_cpu(xpos, ypos, sc);
}

extern "C" int ref_bp_fan_2d_angle_prep(const orc_geom* g, const double* angles, double* xpos,
                                        double* ypos, double* sc)
{
    return FanBackprojection2DAnglePixDrivenPrep(angle_param(g))
        .calculate_on_cpu(angles, xpos, ypos, sc);
}

extern "C" int ref_bp_par_2d_prep(const orc_geom* g, double* xcos, double* ysin)
{
    return ParallelBackprojection2DPixDrivenPrep(par_param(g)).calculate_on_cpu(xcos, ysin,
                                                                                nullptr);
}

extern "C" int ref_fp_par_2d_prep(const orc_geom* g, double* sc, double* bo, int* usex)
{
    return ParallelProjection2DRayDrivenPrepare(fp_param(g)).calculate_on_cpu(sc, bo, usex);
}

extern "C" int ref_fp_par_2d_grad_prep(const orc_geom* g, double* weights, double* pos,
                                       int* usex)
{
    return ParallelProjection2DRayDrivenGradPrep(fp_param(g)).calculate_on_cpu(weights, pos,
                                                                               usex);
}
