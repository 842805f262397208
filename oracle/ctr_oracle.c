/*
 * CPU oracle for the CT reconstruction hot path -- TEST INFRASTRUCTURE ONLY.
 * Geometry preparation (the reference's *Prep::calculate_on_cpu methods) and
 * the float/double instantiations of ctr_oracle_t.h.  See ctr_oracle.h.
 */
#define _USE_MATH_DEFINES
#include <math.h>
#include <stdlib.h>
#include <stddef.h>

#include "ctr_oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef M_PI_4
#define M_PI_4 0.78539816339744830962
#endif

/* src/filter.cc:18-65.  Taps n in [-ns, ns] at filter[n + ns]; type 0 (par)
 * and 2 (flat) share the parallel-beam kernel, type 1 is the equiangular fan
 * kernel; `window` is unused by the reference and absent here. */
int orc_ramp_filter_prep(unsigned ns, double ds, double dsd, int type, double* filter)
{
    double* h = filter + ns;
    const int n = (int)ns;
    if (type == 0 || type == 2) {
        const double ds2_inv = 1.0 / (ds * ds);
        const double pi2_inv = 1.0 / (M_PI * M_PI);
        for (int k = -n; k <= n; ++k) {
            if (k == 0)
                h[k] = 0.25 * ds2_inv;
            else if (k % 2 == 0)
                h[k] = 0;
            else
                h[k] = -pi2_inv * ds2_inv / (double)(k * k);
        }
        return 1;
    }
    if (type == 1) {
        const double pidsd2_inv = 1.0 / (M_PI * M_PI * dsd * dsd);
        for (int k = -n; k <= n; ++k) {
            if (k == 0) {
                h[k] = 0.25 / (ds * ds);
            } else if (k % 2 == 0) {
                h[k] = 0;
            } else {
                const double sa = sin((double)k * ds / dsd);
                h[k] = -pidsd2_inv / (sa * sa);
            }
        }
        return 1;
    }
    return 0;
}

/* Pixel-centre tables shared by the fan preps (src/bp_fan_2d.cc:22-42):
 * positions advance by repeated addition, x to the right, y downwards. */
static void pixel_positions(const orc_geom* g, double* xpos, double* ypos)
{
    const double centx = (double)(g->nx - 1) / 2 + g->offset_x;
    const double centy = (double)(g->ny - 1) / 2 + g->offset_y;
    double posx = -centx * g->dx, posy = centy * g->dy;
    for (unsigned ix = 0; ix < g->nx; ++ix) {
        xpos[ix] = posx;
        posx += g->dx;
    }
    for (unsigned iy = 0; iy < g->ny; ++iy) {
        ypos[iy] = posy;
        posy -= g->dy;
    }
}

/* src/bp_fan_2d.cc:18-44: view angles by repeated addition of orbit */
int orc_bp_fan_2d_prep(const orc_geom* g, double* xpos, double* ypos, double* sincostbl)
{
    double angle = g->orbit_start;
    for (unsigned ia = 0; ia < g->na; ++ia) {
        sincostbl[2 * ia] = sin(angle);
        sincostbl[2 * ia + 1] = cos(angle);
        angle += g->orbit;
    }
    pixel_positions(g, xpos, ypos);
    return 1;
}

/* src/bp_fan_2d_angle.cc:18-45 (the grad prep of the reference leaves ypos
 * uninitialised, src/bp_fan_2d_angle.cc:108; this prep serves both) */
int orc_bp_fan_2d_angle_prep(const orc_geom* g, const double* angles, double* xpos,
                             double* ypos, double* sincostbl)
{
    for (unsigned ia = 0; ia < g->na; ++ia) {
        sincostbl[2 * ia] = sin(angles[ia]);
        sincostbl[2 * ia + 1] = cos(angles[ia]);
    }
    pixel_positions(g, xpos, ypos);
    return 1;
}

/* src/bp_par_2d.cc:18-49 (also src/bp_par_2d_sv.cc:19-50) */
int orc_bp_par_2d_prep(const orc_geom* g, double* xcos, double* ysin)
{
    const double centx = (double)(g->nx - 1) / 2 + g->offset_x;
    const double centy = (double)(g->ny - 1) / 2 + g->offset_y;
    double angle = g->orbit_start;
    for (unsigned ia = 0; ia < g->na; ++ia) {
        const double sa = sin(angle), ca = cos(angle);
        double posx = -centx * g->dx;
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            xcos[ia + (size_t)ix * g->na] = posx * ca;
            posx += g->dx;
        }
        double posy = centy * g->dy;
        for (unsigned iy = 0; iy < g->ny; ++iy) {
            ysin[ia + (size_t)iy * g->na] = posy * sa;
            posy -= g->dy;
        }
        angle += g->orbit;
    }
    return 1;
}

static int views_along_x(double angle)
{
    return !((angle >= M_PI_4 && angle < 3 * M_PI_4) ||
             (angle >= 5 * M_PI_4 && angle < 7 * M_PI_4));
}

/* src/fp_par_2d.cc:149-208: the running angle is wrapped into [0, 2pi) */
int orc_fp_par_2d_prep(const orc_geom* g, double* sincostbl, double* beginoffset, int* usex)
{
    const double centx = (double)(g->nx - 1) / 2.0 + g->offset_x;
    const double centy = (double)(g->ny - 1) / 2.0 + g->offset_y;
    const double cents = (double)(g->ns - 1) / 2.0 + g->offset_s;
    double angle = g->orbit_start;
    for (unsigned ia = 0; ia < g->na; ++ia) {
        while (angle < 0) angle += 2 * M_PI;
        while (angle >= 2 * M_PI) angle -= 2 * M_PI;
        const double sa = sin(angle), ca = cos(angle);
        sincostbl[2 * ia] = sa;
        sincostbl[2 * ia + 1] = ca;
        usex[ia] = views_along_x(angle);
        double step, chan, begin;
        if (usex[ia]) {
            step = g->dy * sa / (ca * g->dx);
            chan = g->ds / (ca * g->dx);
            begin = centx - centy * step - cents * chan;
        } else {
            step = g->dx * ca / (sa * g->dy);
            chan = -g->ds / (sa * g->dy);
            begin = centy - centx * step - cents * chan;
        }
        double* bo = beginoffset + (size_t)ia * g->ns * 2;
        for (unsigned is = 0; is < g->ns; ++is) {
            bo[2 * is] = begin;
            bo[2 * is + 1] = step;
            begin += chan;
        }
        angle += g->orbit;
    }
    return 1;
}

/* src/fp_par_2d.cc:18-80: ray casting.  The view angle and the channel's
 * detector coordinate are running sums (angle += orbit, s += ds), the angle
 * is not wrapped, and a ray takes (int)(chord / step) samples of step
 * step_size (pixels) from its entry point on the FoV circle of radius fov;
 * a ray that misses the circle has none. */
int orc_fp_par_2d_cast_prep(const orc_geom* g, double step_size, double* sincostbl, double* begins,
                            int* nsteps)
{
    const double xc = (double)(g->nx - 1) / 2.0 + g->offset_x;
    const double yc = (double)(g->ny - 1) / 2.0 + g->offset_y;
    const double fov2 = g->fov * g->fov;
    const double s0 = -((double)(g->ns - 1) / 2.0 + g->offset_s) * g->ds;
    double angle = g->orbit_start;
    for (unsigned ia = 0; ia < g->na; ++ia) {
        const double sa = sin(angle), ca = cos(angle);
        sincostbl[2 * ia] = sa;
        sincostbl[2 * ia + 1] = ca;
        const double sx = step_size * sa, sy = step_size * ca;
        const int along_x = sa > (1.0 / 1.414);
        double s = s0;
        for (unsigned is = 0; is < g->ns; ++is) {
            const size_t r = (size_t)ia * g->ns + is;
            const double h2 = fov2 - s * s;
            if (h2 > 0) {
                const double h = sqrt(h2);
                const double x1 = (s * ca - h * sa) / g->dx + xc;
                const double y1 = -(s * sa + h * ca) / g->dy + yc;
                const double x2 = (s * ca + h * sa) / g->dx + xc;
                const double y2 = -(s * sa - h * ca) / g->dy + yc;
                nsteps[r] = along_x ? (int)((x2 - x1) / sx) : (int)((y2 - y1) / sy);
                begins[2 * r] = x1;
                begins[2 * r + 1] = y1;
            } else {
                nsteps[r] = 0;
                begins[2 * r] = 0;
                begins[2 * r + 1] = 0;
            }
            s += g->ds;
        }
        angle += g->orbit;
    }
    return 1;
}

/* src/fp_par_2d.cc:396-452: distance driven.  The running angle is wrapped
 * into [0, 2pi); per channel (footprint centre, step per line, half width),
 * the centre a running sum over channels. */
int orc_fp_par_2d_dd_prep(const orc_geom* g, double* sincostbl, double* beginoffset, int* usex)
{
    const double centx = (double)(g->nx - 1) / 2.0 + g->offset_x;
    const double centy = (double)(g->ny - 1) / 2.0 + g->offset_y;
    const double cents = (double)(g->ns - 1) / 2.0 + g->offset_s;
    double angle = g->orbit_start;
    for (unsigned ia = 0; ia < g->na; ++ia) {
        while (angle < 0) angle += 2 * M_PI;
        while (angle >= 2 * M_PI) angle -= 2 * M_PI;
        const double sa = sin(angle), ca = cos(angle);
        sincostbl[2 * ia] = sa;
        sincostbl[2 * ia + 1] = ca;
        usex[ia] = views_along_x(angle);
        double step, chan, begin;
        if (usex[ia]) {
            step = g->dy * sa / (ca * g->dx);
            chan = g->ds / (ca * g->dx);
            begin = centx - centy * step - cents * chan;
        } else {
            step = g->dx * ca / (sa * g->dy);
            chan = -g->ds / (sa * g->dy);
            begin = centy - centx * step - cents * chan;
        }
        double* bo = beginoffset + (size_t)ia * g->ns * 3;
        for (unsigned is = 0; is < g->ns; ++is) {
            bo[3 * is] = begin;
            bo[3 * is + 1] = step;
            bo[3 * is + 2] = chan / 2;
            begin += chan;
        }
        angle += g->orbit;
    }
    return 1;
}

/* src/fp_par_2d.cc:547-596: the angle is NOT wrapped (as in the reference);
 * per view n = nx = ny (channel of the line's first pixel, channel step). */
int orc_fp_par_2d_dd_grad_prep(const orc_geom* g, double* weights, double* pos, int* usex)
{
    const double centx = (double)(g->nx - 1) / 2.0 + g->offset_x;
    const double centy = (double)(g->ny - 1) / 2.0 + g->offset_y;
    const double cents = (double)(g->ns - 1) / 2.0 + g->offset_s;
    double angle = g->orbit_start;
    for (unsigned ia = 0; ia < g->na; ++ia) {
        const double sa = sin(angle), ca = cos(angle);
        const int ux = views_along_x(angle);
        usex[ia] = ux;
        double begin, o1, o2;
        unsigned n;
        if (ux) {
            weights[ia] = fabs(g->dy / ca);
            o1 = g->dx * ca / g->ds;
            o2 = -g->dy * sa / g->ds;
            begin = cents - centx * o1 - centy * o2;
            n = g->ny;
        } else {
            weights[ia] = fabs(g->dx / sa);
            o1 = -g->dy * sa / g->ds;
            o2 = g->dx * ca / g->ds;
            begin = cents - centy * o1 - centx * o2;
            n = g->nx;
        }
        double* pp = pos + (size_t)ia * g->nx * 2;
        for (unsigned i = 0; i < n; ++i) {
            pp[2 * i] = begin;
            pp[2 * i + 1] = o1;
            begin += o2;
        }
        angle += g->orbit;
    }
    return 1;
}

/* src/fp_par_2d.cc:285-321: the angle is NOT wrapped here (as in the
 * reference); pos holds, per view, n = nx = ny (channel start, channel step)
 * pairs. */
int orc_fp_par_2d_grad_prep(const orc_geom* g, double* weights, double* pos, int* usex)
{
    const double centx = (double)(g->nx - 1) / 2.0 + g->offset_x;
    const double centy = (double)(g->ny - 1) / 2.0 + g->offset_y;
    const double cents = (double)(g->ns - 1) / 2.0 + g->offset_s;
    double angle = g->orbit_start;
    double* pp = pos;
    for (unsigned ia = 0; ia < g->na; ++ia) {
        const double sa = sin(angle), ca = cos(angle);
        usex[ia] = views_along_x(angle);
        if (usex[ia]) {
            weights[ia] = fabs(g->dy / ca);
            const double o1 = g->dx * ca / g->ds;
            const double o2 = -g->dy * sa / g->ds;
            double begin = cents - centx * o1 - centy * o2;
            for (unsigned iy = 0; iy < g->ny; ++iy) {
                pp[0] = begin;
                pp[1] = o1;
                begin += o2;
                pp += 2;
            }
        } else {
            weights[ia] = fabs(g->dx / sa);
            const double o1 = -g->dy * sa / g->ds;
            const double o2 = g->dx * ca / g->ds;
            double begin = cents - centy * o1 - centx * o2;
            for (unsigned ix = 0; ix < g->nx; ++ix) {
                pp[0] = begin;
                pp[1] = o1;
                begin += o2;
                pp += 2;
            }
        }
        angle += g->orbit;
    }
    return 1;
}

/* ---- helical rebinning helpers (src/helical_interpolation.cc:80-334) ---- */

/* Slice z position: z0 plus dz added iz times, as the calculate_on_cpu loops
 * advance it (src/helical_interpolation.cc:339-347). */
static double heli_slice_z(const orc_heli* h, unsigned iz)
{
    double z = h->z0;
    for (unsigned i = 0; i < iz; ++i) z += h->dz;
    return z;
}

/* Detector rows [*r0, *r1) averaged for one sample whose source sits z_dif
 * below the slice, with cos(gamma) = cg: the thick-slice edges projected onto
 * the detector (src/helical_interpolation.cc:105-111), clamped to the
 * detector.  Returns 0 when the slab misses the detector (bottom edge above
 * row 0 or top edge past the last row). */
static int heli_rows(const orc_heli* h, double center_t, double z_dif, double cg, int* r0, int* r1)
{
    double top = center_t - (z_dif + h->thickness / 2.0) / h->dso * cg * h->dsd;
    double bot = center_t - (z_dif - h->thickness / 2.0) / h->dso * cg * h->dsd;
    if (bot < 0 || top >= (double)h->nt) return 0;
    if (top < 0) top = 0;
    if (bot >= (double)h->nt) bot = (double)h->nt;
    *r0 = (int)floor(top);
    *r1 = (int)ceil(bot);
    return 1;
}

#define T float
#define SFX f32
#include "ctr_oracle_t.h"
#undef T
#undef SFX

#define T double
#define SFX f64
#include "ctr_oracle_t.h"
#undef T
#undef SFX
